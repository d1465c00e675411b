// Blocked Cholesky factorisation, triangular solves, the exact residual and the
// refinement driver behind qmlg_solve.
//
// Restates fcho_solve (qml/fcho_solve.f90:23-52): dpotrf("U") then dpotrs("U",
// nrhs=1) on a column-major matrix.  Kernels work on the row-major view of the
// same memory, R[i][j] = A[j + i*lda]: the column-major upper triangle that
// dpotrf("U") factorises is R's lower triangle, so U (A = U^T U) is stored as
// L = U^T in R's lower triangle and R's strictly upper triangle (the column-major
// strictly lower one) keeps the original matrix, as LAPACK leaves it.
//
// Right-looking blocked algorithm, block NB = 64:
//   potrf_diag   one CTA factorises the NB x NB diagonal block in shared memory
//                (FP64), flagging the first non-positive pivot like LAPACK's info;
//   trsm_panel   the panel below it: X <- X L_kk^-T, one CTA per 64 rows;
//   syrk_update  the trailing lower triangle: C <- C - P P^T with 64 x 64 tiles.
// After a failed pivot every later kernel sees the info flag and returns.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include <cooperative_groups.h>

#include "common.cuh"
#include "emulated_gemm.cuh"
#include "rsqrt.cuh"
#include "exact_acc.cuh"

namespace cg = cooperative_groups;

namespace {

constexpr int NB = 64;

// ---------------------------------------------------------------- factor --

// 1/sqrt(p) for a positive finite double, with as few FP64 instructions as possible
// (on this GPU each costs ~64 cycles of the FP64 pipe; sqrt and division ~650): an
// Number of lower-triangle elements (r, s) with c < s <= r < NB.
__host__ __device__ constexpr int tri_prefix(int c) { return (NB - 1 - c) * (NB - c) / 2; }

constexpr int POTRF_THREADS = 256;
// Warps 0-2 and 4-6 update; lane 0 of warp 3 takes the pivots, alone on its
// scheduler's FP64 pipe (warp 7 only joins the barriers).
constexpr int POTRF_WORKERS = 192;
constexpr int POTRF_PIVOT = 96;

// Pivot of column c: rd[c] <- 1/sqrt(S_cc) (> 0), rd2[c] <- 1/S_cc; S_cc keeps the
// pivot (the factor's diagonal sqrt(S_cc) = S_cc rd[c] is formed at write-back).
// When S_cc is not positive and finite, rd[c] <- 0 marks the failure and the failing
// column is recorded in info.  The checks are on the bits (no FP64 compares).
__device__ __forceinline__ void potrf_pivot(double (*S)[NB + 1], double *rd, double *rd2, int c,
                                            int k0, int nb, int *info)
{
    const double p = S[c][c];
    const long long b = __double_as_longlong(p);
    if (b <= 0 || ((unsigned long long)b >> 52) >= 0x7ffull) {
        if (c < nb) atomicCAS(info, 0, k0 + c + 1);
        rd[c] = 0.0;
        return;
    }
    const double y = rsqrt_halley(p);
    rd[c] = y;
    rd2[c] = y * y;
}

// Barrier of the 192 worker threads only (the pivot warp does not wait for it).
__device__ __forceinline__ void potrf_workers_sync()
{
    asm volatile("bar.sync 1, 192;" ::: "memory");
}

__device__ __forceinline__ void potrf_diag_block(double *__restrict__ A, int64_t lda, int n, int k0,
                                                 double shift, int *__restrict__ info)
{
    // Right-looking in shared memory.  One FP64 warp instruction occupies a
    // scheduler's FP64 pipe for ~64 cycles whatever its active lanes, so the
    // update is laid out for dense warps and one FMA per element.  Phase c: warps
    // 0 and 4 scale column c (lc[r] = S_rc / S_cc, with rd2[c] = 1/S_cc), the workers
    // meet at their own barrier, then every element with c < s <= r takes
    // S_rs -= lc[r] S_sc.  The elements are listed in `order` by s descending, r
    // descending, so phase c's are the first tri_prefix(c) entries and the last of
    // them is the next diagonal S_{c+1,c+1}: the workers take the others in turn
    // (each issues the next element's loads before this one's store), while the
    // pivot thread updates that diagonal and takes its pivot at once, so the pivot
    // latency overlaps the updates.  rd[c] is written one phase before it is read,
    // so rd[c] == 0 is a race-free failure signal.  Columns are scaled by rd at
    // write-back.
    __shared__ double S[NB][NB + 1];
    __shared__ double rd[NB], rd2[NB], lc[NB];
    __shared__ unsigned short order[tri_prefix(0)];
    if (*info != 0) return;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nb = min(NB, n - k0);
#pragma unroll
    for (int e = tid; e < NB * NB; e += POTRF_THREADS) {  // loads issued back to back
        const int r = e >> 6, c = e & 63;
        double v = (r == c) ? 1.0 : 0.0;  // identity padding keeps short blocks regular
        if (r < nb && c <= r) {
            v = A[(int64_t)(k0 + r) * lda + (k0 + c)];
            if (r == c) v += shift;
        }
        S[r][c] = v;
    }
    if (tid >= 1 && tid < NB) {
        const int sc = tid, base = tri_prefix(sc);
        for (int t = 0; t < NB - sc; ++t) order[base + t] = (unsigned short)(((NB - 1 - t) << 8) | sc);
    }
    __syncthreads();
    if (tid == POTRF_PIVOT) potrf_pivot(S, rd, rd2, 0, k0, nb, info);
    __syncthreads();
    const bool worker = warp != 3 && warp != 7;
    const int wid = (warp < 3 ? warp : warp - 1) * 32 + lane;
    for (int c = 0; c + 1 < NB; ++c) {
        if (__double_as_longlong(rd[c]) == 0) return;
        const double y2 = rd2[c];
        if (tid == POTRF_PIVOT) {
            const double v = S[c + 1][c];
            S[c + 1][c + 1] = fma(-v * y2, v, S[c + 1][c + 1]);
            potrf_pivot(S, rd, rd2, c + 1, k0, nb, info);
        } else if (worker) {
            if (warp == 0 || warp == 4) {
                const int r = c + 1 + lane + (warp == 4 ? 32 : 0);
                if (r < NB) lc[r] = S[r][c] * y2;
            }
            potrf_workers_sync();
            const int cnt = tri_prefix(c) - 1;
            int e = wid, r = 0, sc = 0;
            double x = 0.0, a = 0.0, b = 0.0;
            if (e < cnt) {
                const unsigned code = order[e];
                r = (int)(code >> 8);
                sc = (int)(code & 255u);
                x = S[r][sc];
                a = lc[r];
                b = S[sc][c];
            }
            while (e < cnt) {
                const int en = e + POTRF_WORKERS;
                int rn = 0, sn = 0;
                double xn = 0.0, an = 0.0, bn = 0.0;
                if (en < cnt) {
                    const unsigned code = order[en];
                    rn = (int)(code >> 8);
                    sn = (int)(code & 255u);
                    xn = S[rn][sn];
                    an = lc[rn];
                    bn = S[sn][c];
                }
                S[r][sc] = fma(-a, b, x);
                e = en;
                r = rn;
                sc = sn;
                x = xn;
                a = an;
                b = bn;
            }
        }
        __syncthreads();
    }
    if (__double_as_longlong(rd[NB - 1]) == 0) return;
    for (int e = tid; e < nb * NB; e += blockDim.x) {
        const int r = e >> 6, c = e & 63;
        if (c <= r) A[(int64_t)(k0 + r) * lda + (k0 + c)] = S[r][c] * rd[c];
    }
}

__global__ void __launch_bounds__(POTRF_THREADS)
potrf_diag_kernel(double *__restrict__ A, int64_t lda, int n, int k0, double shift,
                  int *__restrict__ info)
{
    potrf_diag_block(A, lda, n, k0, shift, info);
}

constexpr int TRSM_MAX_ROWS = 128;  // rows per CTA: 4 threads per row

// Rows per TRSM CTA for `rows` rows on `sms` SMs: a multiple of 8 up to 128, chosen
// so the CTAs spread evenly (every SM gets the same number, up to rounding).
inline int trsm_rows_per_cta(int rows, int sms)
{
    sms = std::max(1, sms);
    const int k = (int)qmlg::ceil_div(rows, sms * TRSM_MAX_ROWS);  // CTAs per SM
    const int r = (int)qmlg::ceil_div(qmlg::ceil_div(rows, std::max(1, k * sms)), 8) * 8;
    return std::min(TRSM_MAX_ROWS, std::max(32, r));
}

inline size_t trsm_smem(int rpc) { return (size_t)rpc * (NB + 8) * sizeof(__nv_bfloat16); }

// X <- X L_kk^{-T} for the rows below the diagonal block, blockDim / 4 rows per CTA.
// A row is held by the four lanes of a quad (lane q owns the columns = q mod 4, in
// registers); column c is finished by its owner and broadcast with a shuffle, so
// the substitution needs no block barrier.  With `digits`, the kernel also writes
// what slice_rows would make of the solved rows (the operand of the emulated K = 64
// update that follows): per-row exponents and the `slices` balanced base-128 digit
// planes, digits[s][row][64] with row = global row - (k0 + 64), for the rows below
// drows (zeros past the matrix).
__device__ __forceinline__ void trsm_panel_rows(double *__restrict__ A, int64_t lda, int n, int k0,
                                                const int *__restrict__ info, int slices, int rpad,
                                                int drows, __nv_bfloat16 *__restrict__ digits,
                                                int *__restrict__ expo, int bid)
{
    __shared__ double L[NB][NB + 1];
    __shared__ double rdg[NB];
    extern __shared__ __align__(16) unsigned char trsm_dyn[];
    __nv_bfloat16(*P)[NB + 8] = reinterpret_cast<__nv_bfloat16(*)[NB + 8]>(trsm_dyn);
    if (*info != 0) return;
    const int tid = threadIdx.x, lane = tid & 31;
    const int rpc = blockDim.x >> 2;
    const int nb = min(NB, n - k0);
    const int r1 = k0 + nb, nrows = n - r1;
    const int rbase = bid * rpc;
#pragma unroll 8
    for (int e = tid; e < NB * NB; e += blockDim.x) {
        const int r = e >> 6, c = e & 63;
        L[r][c] = (r < nb && c <= r) ? A[(int64_t)(k0 + r) * lda + (k0 + c)] : (r == c ? 1.0 : 0.0);
    }
    __syncthreads();
    if (tid < NB) rdg[tid] = 1.0 / L[tid][tid];
    const int r = tid >> 2, s0 = tid & 3, qbase = lane & ~3;
    const int grow = rbase + r;
    const bool live = grow < nrows;
    double *row = A + (int64_t)(r1 + (live ? grow : 0)) * lda + k0;
    double x[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = live ? row[s0 + 4 * j] : 0.0;
    __syncthreads();
#pragma unroll
    for (int c = 0; c < NB; ++c) {
        const int jc = c >> 2, oc = c & 3;
        const double t = x[jc] * rdg[c];
        const double xc = __shfl_sync(0xffffffffu, t, qbase | oc);
        if (s0 == oc) x[jc] = xc;
        if (s0 > oc) x[jc] = fma(-xc, L[s0 + 4 * jc][c], x[jc]);
#pragma unroll
        for (int j = jc + 1; j < 16; ++j) x[j] = fma(-xc, L[s0 + 4 * j][c], x[j]);
    }
    if (live)
#pragma unroll
        for (int j = 0; j < 16; ++j) row[s0 + 4 * j] = x[j];
    if (digits == nullptr) return;
    // max |x| on the bits and the power-of-two scaling on the exponent field, as in
    // slice_rows (no FP64 instruction unless an entry is subnormal)
    unsigned long long mb = 0ull;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const unsigned long long bv = (unsigned long long)__double_as_longlong(x[j]) & 0x7fffffffffffffffull;
        mb = bv > mb ? bv : mb;
    }
#pragma unroll
    for (int off = 1; off <= 2; off <<= 1) {
        const unsigned long long o = __shfl_xor_sync(0xffffffffu, mb, off);
        mb = o > mb ? o : mb;
    }
    const double m = __longlong_as_double((long long)mb);
    int e = 0;
    if (m > 0.0 && isfinite(m)) {
        frexp(m, &e);
        e += 1;  // |x| * 2^-e < 1/2
    }
    const int ks = 7 * slices - e;
    long long q[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) {
        const unsigned long long bv = (unsigned long long)__double_as_longlong(x[j]);
        const int E = (int)((bv >> 52) & 0x7ff);
        long long qv = 0;
        if (E == 0) {
            if ((bv & 0x000fffffffffffffull) != 0ull) qv = __double2ll_rn(x[j] * scalbn(1.0, ks));
        } else if (E + ks > 0) {
            qv = __double2ll_rn(__longlong_as_double((long long)(bv + ((unsigned long long)(long long)ks << 52))));
        }
        q[j] = qv;
    }
    if (s0 == 0 && grow < drows) expo[grow] = e;
    const int64_t plane = (int64_t)rpad * NB;
    for (int sl = slices - 1; sl >= 0; --sl) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            // the most significant digit keeps the remainder (|q| <= 64 there)
            const long long d = sl > 0 ? ((q[j] + 64) & 127) - 64 : q[j];
            q[j] = (q[j] - d) >> 7;
            P[r][s0 + 4 * j] = __int2bfloat16_rn((int)d);
        }
        __syncthreads();
        for (int i = tid; i < rpc * (NB / 8); i += blockDim.x) {
            const int rr = i >> 3, ch = i & 7, g = rbase + rr;
            if (g < drows)
                *reinterpret_cast<uint4 *>(digits + sl * plane + (int64_t)g * NB + ch * 8) =
                    *reinterpret_cast<const uint4 *>(&P[rr][ch * 8]);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(4 * TRSM_MAX_ROWS)
trsm_panel_kernel(double *__restrict__ A, int64_t lda, int n, int k0,
                  const int *__restrict__ info, int slices, int rpad, int drows,
                  __nv_bfloat16 *__restrict__ digits, int *__restrict__ expo)
{
    trsm_panel_rows(A, lda, n, k0, info, slices, rpad, drows, digits, expo, blockIdx.x);
}

// Launches the TRSM of the rows below diagonal block k0 (with `digits`: the digit
// planes of the rows below drows as well).
int launch_trsm(double *A, int64_t lda, int n, int k0, const int *d_info, int slices, int rpad,
                int drows, __nv_bfloat16 *digits, int *expo, cudaStream_t s)
{
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(trsm_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)trsm_smem(TRSM_MAX_ROWS));
    });
    if (attr != cudaSuccess) return qmlg::set_cuda_error(attr);
    const int rows = digits != nullptr ? drows : n - (k0 + NB);
    if (rows <= 0) return QMLG_OK;
    const int rpc = trsm_rows_per_cta(rows, qmlg::tc_sm_count());
    trsm_panel_kernel<<<(unsigned)qmlg::ceil_div(rows, rpc), 4 * rpc, trsm_smem(rpc), s>>>(
        A, lda, n, k0, d_info, slices, rpad, drows, digits, expo);
    qmlg::count_launches(1);
    return QMLG_OK;
}

__device__ __forceinline__ void tri_index(int64_t t, int &bi, int &bj)
{
    int64_t r = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > t) --r;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    bi = (int)r;
    bj = (int)(t - r * (r + 1) / 2);
}

// C[i][j] -= sum_t P[i][t] P[j][t] over the trailing lower triangle, FP64.
__global__ void __launch_bounds__(256)
syrk_update_kernel(double *__restrict__ A, int64_t lda, int n, int k0,
                   const int *__restrict__ info)
{
    __shared__ double Ps[16][64 + 1];
    __shared__ double Qs[16][64 + 1];
    if (*info != 0) return;
    const int k1 = k0 + NB;
    int bi, bj;
    tri_index(blockIdx.x, bi, bj);
    const int i0 = k1 + bi * 64, j0 = k1 + bj * 64;
    const int tid = threadIdx.x;
    const int tx = tid & 15, ty = tid >> 4;  // tx -> j (contiguous), ty -> i
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
    for (int t0 = 0; t0 < NB; t0 += 16) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int e = tid + q * 256;
            const int r = e >> 4, c = e & 15;
            const int ri = i0 + r, rj = j0 + r;
            Ps[c][r] = ri < n ? A[(int64_t)ri * lda + k0 + t0 + c] : 0.0;
            Qs[c][r] = rj < n ? A[(int64_t)rj * lda + k0 + t0 + c] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            double pv[4], qv[4];
#pragma unroll
            for (int b = 0; b < 4; ++b) pv[b] = Ps[c][ty + 16 * b];
#pragma unroll
            for (int a = 0; a < 4; ++a) qv[a] = Qs[c][tx + 16 * a];
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] = fma(pv[b], qv[a], acc[a][b]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
        const int i = i0 + ty + 16 * b;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const int j = j0 + tx + 16 * a;
            if (i < n && j < n && j <= i) {
                double *p = A + (int64_t)i * lda + j;
                *p -= acc[a][b];
            }
        }
    }
}


// ------------------------------------------------------------- residual --

constexpr int RES_ROWS = 64;
constexpr int RES_CHUNK = 1024;

// Partial row sums of the symmetric matrix held in R's strictly upper triangle plus
// diag, times x: one CTA per (64 rows, 1024 columns), each product added exactly
// into a 256-bit fixed-point accumulator (exact_acc.cuh).
//  * x's 1024 entries are split once, at the start, into shared memory.
//  * The 64 x 64 tiles of the symmetric matrix are copied into shared memory with
//    cp.async, two buffers deep, so the next tile's loads run under this tile's
//    products.  Element (r, c) sits at r * 64 + (c ^ (r & 31)): row-wise and
//    column-wise stores and the column reads below are all free of bank conflicts.
//  * Warp w takes rows 32 (w & 1) .. +31 (a lane per row) and the column quarter
//    w >> 1 of every tile, so all lanes of a warp meet the same x_j at once: x's
//    sign and split are warp-uniform, and for a matrix without negative entries (a
//    kernel matrix) so is the sign of every product.
//  * The four quarter sums of a row are combined exactly at the end.
struct AccPart {
    unsigned long long l0, l1, l2, l3;
    int f, bad;
};

constexpr int RES_TILE = 64 * 64;  // doubles per tile buffer
constexpr size_t RES_SMEM = 2 * RES_TILE * sizeof(double) + RES_CHUNK * (sizeof(uint2) + sizeof(short));

__device__ __forceinline__ void cp_async8(double *dst, const double *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
}

// Copies the symmetric tile (rows i0.., columns j0..) into T (swizzled, zeros outside).
__device__ __forceinline__ void res_stage(double *T, const double *__restrict__ A, int64_t lda, int n,
                                          const double *__restrict__ diag, int i0, int j0, int tid)
{
    // the two loops write disjoint elements: (j >= i or outside) / (j < i inside)
    for (int e = tid; e < RES_TILE; e += 256) {
        const int rr = e >> 6, c = e & 63;
        const int i = i0 + rr, j = j0 + c;
        double *dst = T + rr * 64 + (c ^ (rr & 31));
        if (i < n && j < n) {
            if (j > i) cp_async8(dst, A + (int64_t)i * lda + j);
            else if (j == i) cp_async8(dst, diag + i);
        } else {
            *dst = 0.0;
        }
    }
    for (int e = tid; e < RES_TILE; e += 256) {
        // lower part from the transposed upper tile: R[j][i] for j < i
        const int c = e >> 6, rr = e & 63;
        const int i = i0 + rr, j = j0 + c;
        if (i < n && j < n && j < i) cp_async8(T + rr * 64 + (c ^ (rr & 31)), A + (int64_t)j * lda + i);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

__device__ __forceinline__ void symv_exact_partial_block(const double *__restrict__ A, int64_t lda,
                                                         int n, const double *__restrict__ diag,
                                                         const double *__restrict__ x,
                                                         AccPart *__restrict__ partial, int bx,
                                                         int by)
{
    extern __shared__ __align__(16) unsigned char res_smem[];
    double *T = reinterpret_cast<double *>(res_smem);                         // [2][RES_TILE]
    uint2 *xs = reinterpret_cast<uint2 *>(T + 2 * RES_TILE);                  // low 32 bits; high 21 | sign << 31
    short *xe = reinterpret_cast<short *>(xs + RES_CHUNK);                    // exponent - 2150
    __shared__ int xbad;
    static_assert(RES_TILE * sizeof(double) >= 256 * sizeof(AccPart), "the combine reuses a tile buffer");
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int i0 = bx * RES_ROWS;
    const int c0 = by * RES_CHUNK;
    const int ntiles = (min(n, c0 + RES_CHUNK) - c0 + 63) / 64;
    const int r = lane + 32 * (warp & 1), cq = 16 * (warp >> 1), sw = r & 31;
    res_stage(T, A, lda, n, diag, i0, c0, tid);
    if (tid == 0) xbad = 0;
    __syncthreads();
    for (int t = tid; t < RES_CHUNK; t += 256) {
        const unsigned long long u =
            (unsigned long long)__double_as_longlong((c0 + t < n) ? x[c0 + t] : 0.0);
        const uint32_t hw = (uint32_t)(u >> 32), ef = (hw >> 20) & 0x7ffu;
        xs[t] = make_uint2((uint32_t)u, (hw & 0x800fffffu) | (ef ? 0x100000u : 0u));
        xe[t] = (short)((int)(ef ? ef : 1u) - 2 * 1075);
        if (ef == 0x7ffu) xbad = 1;
    }
    qmlg::Acc acc;
    qmlg::acc_init(acc);
    for (int k = 0; k < ntiles; ++k) {
        if (k + 1 < ntiles) {
            res_stage(T + ((k + 1) & 1) * RES_TILE, A, lda, n, diag, i0, c0 + 64 * (k + 1), tid);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        const double *Tk = T + (k & 1) * RES_TILE + r * 64;
        const uint2 *xk = xs + 64 * k;
        const short *ek = xe + 64 * k;
#pragma unroll 4
        for (int c = cq; c < cq + 16; ++c) {
            const unsigned long long ua = (unsigned long long)__double_as_longlong(Tk[c ^ sw]);
            const uint32_t aw = (uint32_t)(ua >> 32), ef = (aw >> 20) & 0x7ffu;
            const uint2 xb = xk[c];
            unsigned long long hi, lo;
            qmlg::mul53((uint32_t)ua, (aw & 0xfffffu) | (ef ? 0x100000u : 0u), xb.x, xb.y & 0x1fffffu,
                        hi, lo);
            acc.bad |= ef == 0x7ffu;
            qmlg::acc_add_mag_fast(acc, hi, lo, (int)(ef ? ef : 1u) + ek[c], ((aw ^ xb.y) >> 31) != 0u);
        }
        __syncthreads();  // the buffer is refilled by the next iteration's copies
    }
    acc.bad |= xbad;
    // combine the four column quarters of each row (exact, fixed order)
    AccPart *comb = reinterpret_cast<AccPart *>(T);  // [quarter][row]
    {
        AccPart &o = comb[(warp >> 1) * 64 + r];
        o.l0 = acc.l0;
        o.l1 = acc.l1;
        o.l2 = acc.l2;
        o.l3 = acc.l3;
        o.f = acc.f;
        o.bad = acc.bad;
    }
    __syncthreads();
    const int i = i0 + tid;
    if (tid < 64 && i < n) {
        qmlg::Acc a;
        qmlg::acc_init(a);
        for (int q = 0; q < 4; ++q) {
            const AccPart &p = comb[q * 64 + tid];
            qmlg::Acc b;
            b.l0 = p.l0;
            b.l1 = p.l1;
            b.l2 = p.l2;
            b.l3 = p.l3;
            b.f = p.f;
            b.bad = p.bad;
            qmlg::acc_add_acc(a, b);
        }
        AccPart &o = partial[(int64_t)by * n + i];
        o.l0 = a.l0;
        o.l1 = a.l1;
        o.l2 = a.l2;
        o.l3 = a.l3;
        o.f = a.f;
        o.bad = a.bad;
    }
}

// Opt-in to the residual's dynamic shared memory (once per process and kernel).
template <typename K>
int res_smem_attr(K kernel)
{
    const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)RES_SMEM);
    return e == cudaSuccess ? QMLG_OK : qmlg::set_cuda_error(e);
}

__global__ void __launch_bounds__(256)
symv_exact_partial_kernel(const double *__restrict__ A, int64_t lda, int n,
                          const double *__restrict__ diag, const double *__restrict__ x,
                          AccPart *__restrict__ partial)
{
    symv_exact_partial_block(A, lda, n, diag, x, partial, blockIdx.x, blockIdx.y);
}

// r[i] = y[i] - lambda x[i] - sum_chunks partial, summed exactly, rounded once.
__device__ __forceinline__ void residual_finish_block(const AccPart *__restrict__ partial,
                                                      int nchunks, int n, double lambda,
                                                      const double *__restrict__ x,
                                                      const double *__restrict__ y,
                                                      double *__restrict__ r, int bid)
{
    const int i = bid * blockDim.x + threadIdx.x;
    if (i >= n) return;
    qmlg::Acc a;
    qmlg::acc_init(a);
    qmlg::acc_add_prod(a, y[i], 1.0);
    qmlg::acc_add_prod(a, lambda, x[i], true);
    for (int c = 0; c < nchunks; ++c) {
        const AccPart p = partial[(int64_t)c * n + i];
        qmlg::Acc b;
        b.l0 = p.l0;
        b.l1 = p.l1;
        b.l2 = p.l2;
        b.l3 = p.l3;
        b.f = p.f;
        b.bad = p.bad;
        qmlg::acc_add_acc(a, b, true);
    }
    r[i] = qmlg::acc_to_double(a);
}

__global__ void residual_finish_kernel(const AccPart *__restrict__ partial, int nchunks, int n,
                                       double lambda, const double *__restrict__ x,
                                       const double *__restrict__ y, double *__restrict__ r)
{
    residual_finish_block(partial, nchunks, n, lambda, x, y, r, blockIdx.x);
}

// ---------------------------------------------------------------- vectors --

__global__ void copy_diag_kernel(const double *__restrict__ A, int64_t lda, int n,
                                 double *__restrict__ d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = A[(int64_t)i * lda + i];
}

__device__ __forceinline__ void axpy_norms_block(double *__restrict__ x,
                                                 const double *__restrict__ dx, int n,
                                                 double *__restrict__ sums, int bid)
{
    // x += dx; sums[0] += |dx|^2, sums[1] += |x|^2 (block partials, then atomics)
    __shared__ double s0[8], s1[8];
    const int i = bid * blockDim.x + threadIdx.x;
    double a = 0.0, b = 0.0;
    if (i < n) {
        const double d = dx[i];
        const double v = x[i] + d;
        x[i] = v;
        a = d * d;
        b = v * v;
    }
    for (int off = 16; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b += __shfl_xor_sync(0xffffffffu, b, off);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s0[w] = a;
        s1[w] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ta = 0.0, tb = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            ta += s0[k];
            tb += s1[k];
        }
        atomicAdd(&sums[0], ta);
        atomicAdd(&sums[1], tb);
    }
}

__global__ void axpy_norms_kernel(double *__restrict__ x, const double *__restrict__ dx, int n,
                                  double *__restrict__ sums)
{
    axpy_norms_block(x, dx, n, sums, blockIdx.x);
}

// ------------------------------------------- cooperative triangular solves --
//
// One cooperative launch per triangular solve; grid-wide barriers separate the
// 64-row block steps.  Step kb: CTA 0 applies block kb-1's solution to the rows of
// block kb and solves the diagonal block with one warp (reciprocal pivots), while
// the other CTAs apply block kb-1's solution to every row below block kb.

constexpr int TRSV_THREADS = 256;

__device__ __forceinline__ void load_diag_block(const double *__restrict__ A, int64_t lda, int k0,
                                                int nb, double (*L)[NB + 1], double *dinv)
{
    for (int e = threadIdx.x; e < NB * NB; e += blockDim.x) {
        const int r = e >> 6, c = e & 63;
        L[r][c] = (r < nb && c <= r) ? A[(int64_t)(k0 + r) * lda + (k0 + c)] : 0.0;
    }
    __syncthreads();
    if (threadIdx.x < NB) dinv[threadIdx.x] = threadIdx.x < nb ? 1.0 / L[threadIdx.x][threadIdx.x] : 0.0;
    __syncthreads();
}

__global__ void __launch_bounds__(TRSV_THREADS)
trsv_fwd_coop_kernel(const double *__restrict__ A, int64_t lda, int n, double *__restrict__ x)
{
    cg::grid_group grid = cg::this_grid();
    __shared__ double L[NB][NB + 1];
    __shared__ double dinv[NB];
    __shared__ double zp[NB];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int nw = TRSV_THREADS / 32;
    const int nblk = (n + NB - 1) / NB;
    for (int kb = 0; kb < nblk; ++kb) {
        const int k0 = kb * NB, nb = min(NB, n - k0), kp = k0 - NB;
        if (kb > 0) {
            if (tid < NB) zp[tid] = x[kp + tid];
            __syncthreads();
        }
        if (blockIdx.x == 0) {
            if (kb > 0) {
                for (int r = warp; r < nb; r += nw) {
                    const double *row = A + (int64_t)(k0 + r) * lda + kp;
                    double sum = fma(row[lane], zp[lane], row[lane + 32] * zp[lane + 32]);
                    for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
                    if (lane == 0) x[k0 + r] -= sum;
                }
            }
            load_diag_block(A, lda, k0, nb, L, dinv);
            if (warp == 0) {
                double v0 = lane < nb ? x[k0 + lane] : 0.0;
                double v1 = lane + 32 < nb ? x[k0 + lane + 32] : 0.0;
                for (int c = 0; c < nb; ++c) {
                    const double own = __shfl_sync(0xffffffffu, c < 32 ? v0 : v1, c & 31);
                    const double zc = own * dinv[c];
                    if (c < 32) {
                        if (lane == c) v0 = zc;
                    } else if (lane == c - 32) {
                        v1 = zc;
                    }
                    if (lane > c) v0 = fma(-L[lane][c], zc, v0);
                    if (lane + 32 > c) v1 = fma(-L[lane + 32][c], zc, v1);
                }
                if (lane < nb) x[k0 + lane] = v0;
                if (lane + 32 < nb) x[k0 + lane + 32] = v1;
            }
        } else if (kb > 0) {
            const int tw = (gridDim.x - 1) * nw;
            for (int r = k0 + NB + (blockIdx.x - 1) * nw + warp; r < n; r += tw) {
                const double *row = A + (int64_t)r * lda + kp;
                double sum = fma(row[lane], zp[lane], row[lane + 32] * zp[lane + 32]);
                for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
                if (lane == 0) x[r] -= sum;
            }
        }
        grid.sync();
    }
}

__global__ void __launch_bounds__(TRSV_THREADS)
trsv_bwd_coop_kernel(const double *__restrict__ A, int64_t lda, int n, double *__restrict__ x)
{
    cg::grid_group grid = cg::this_grid();
    __shared__ double L[NB][NB + 1];
    __shared__ double dinv[NB];
    __shared__ double zp[NB];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nblk = (n + NB - 1) / NB;
    for (int kb = nblk - 1; kb >= 0; --kb) {
        const int k0 = kb * NB, nb = min(NB, n - k0), kn = k0 + NB;
        const int nbn = kb < nblk - 1 ? min(NB, n - kn) : 0;
        if (nbn > 0) {
            if (tid < NB) zp[tid] = tid < nbn ? x[kn + tid] : 0.0;
            __syncthreads();
        }
        if (blockIdx.x == 0) {
            if (nbn > 0 && tid < nb) {
                double sum = 0.0;
                for (int r = 0; r < nbn; ++r) sum = fma(A[(int64_t)(kn + r) * lda + k0 + tid], zp[r], sum);
                x[k0 + tid] -= sum;
            }
            load_diag_block(A, lda, k0, nb, L, dinv);
            if (warp == 0) {
                double v0 = lane < nb ? x[k0 + lane] : 0.0;
                double v1 = lane + 32 < nb ? x[k0 + lane + 32] : 0.0;
                for (int c = nb - 1; c >= 0; --c) {
                    const double own = __shfl_sync(0xffffffffu, c < 32 ? v0 : v1, c & 31);
                    const double xc = own * dinv[c];
                    if (c < 32) {
                        if (lane == c) v0 = xc;
                    } else if (lane == c - 32) {
                        v1 = xc;
                    }
                    if (lane < c) v0 = fma(-L[c][lane], xc, v0);
                    if (lane + 32 < c) v1 = fma(-L[c][lane + 32], xc, v1);
                }
                if (lane < nb) x[k0 + lane] = v0;
                if (lane + 32 < nb) x[k0 + lane + 32] = v1;
            }
        } else if (nbn > 0) {
            const int tt = (gridDim.x - 1) * TRSV_THREADS;
            for (int t = (blockIdx.x - 1) * TRSV_THREADS + tid; t < k0; t += tt) {
                double sum = 0.0;
                for (int r = 0; r < nbn; ++r) sum = fma(A[(int64_t)(kn + r) * lda + t], zp[r], sum);
                x[t] -= sum;
            }
        }
        grid.sync();
    }
}

// Inverse of every 64 x 64 diagonal block of the factor (lower triangular), one CTA
// per block: column c of L_kk^{-1} by forward substitution (thread c).  Blocks of
// a short last block are padded with the identity.
__device__ __forceinline__ void invert_diag_block(const double *__restrict__ A, int64_t lda, int n,
                                                  double *__restrict__ Linv, int kb)
{
    __shared__ double L[NB][NB + 1];
    __shared__ double X[NB][NB + 1];
    const int k0 = kb * NB, nb = min(NB, n - k0);
    const int tid = threadIdx.x;
    for (int e = tid; e < NB * NB; e += blockDim.x) {
        const int r = e >> 6, c = e & 63;
        double v = (r == c) ? 1.0 : 0.0;
        if (r < nb && c <= r) v = A[(int64_t)(k0 + r) * lda + (k0 + c)];
        L[r][c] = v;
    }
    __syncthreads();
    const int c = tid;  // column of the inverse
    for (int r = 0; r < NB; ++r) {
        double v = (r == c) ? 1.0 : 0.0;
        for (int t = c; t < r; ++t) v = fma(-L[r][t], X[t][c], v);
        X[r][c] = (r >= c) ? v / L[r][r] : 0.0;
    }
    __syncthreads();
    double *dst = Linv + (int64_t)kb * NB * NB;
    for (int e = tid; e < NB * NB; e += blockDim.x) dst[e] = X[e >> 6][e & 63];
}

__global__ void __launch_bounds__(64)
invert_diag_blocks_kernel(const double *__restrict__ A, int64_t lda, int n,
                          double *__restrict__ Linv)
{
    invert_diag_block(A, lda, n, Linv, blockIdx.x);
}

// y[0..64) = M v for a 64 x 64 row-major M (M in global memory, v in shared memory);
// 256 threads: row r = tid / 4, quarter tid % 4 of the columns, combined by shuffles.
__device__ __forceinline__ double gemv64_row(const double *__restrict__ M, int64_t ldm,
                                             const double *v, int tid, int rows)
{
    // rows >= `rows` contribute 0 and are not read; every lane runs the shuffles
    const int r = tid >> 2, qq = tid & 3;
    double s = 0.0;
    if (r < rows) {
        const double *row = M + (int64_t)r * ldm + qq * 16;
#pragma unroll
        for (int c = 0; c < 16; ++c) s = fma(row[c], v[qq * 16 + c], s);
    }
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    return s;
}

// y[t] = sum_r M[r][t] v[r] (transposed), same thread layout: t = tid / 4.
__device__ __forceinline__ double gemv64_col(const double *__restrict__ M, int64_t ldm,
                                             const double *v, int tid)
{
    const int t = tid >> 2, qq = tid & 3;
    double s = 0.0;
#pragma unroll
    for (int r = 0; r < 16; ++r) s = fma(M[(int64_t)(qq * 16 + r) * ldm + t], v[qq * 16 + r], s);
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    return s;
}

// Triangular solves with the block inverses, one cooperative launch per direction
// and no flag or fence: each solved entry is its own ready signal.  The output
// vectors are first filled with a signalling-NaN sentinel that no arithmetic result
// carries; a solved entry is stored once with a relaxed store, and a reader polls
// exactly the entries it needs until none is the sentinel.  With the couplings of
// neighbouring blocks
//   M_i = L_ii^-1 L_i,i-1        P_i = (L_i+1,i L_ii^-1)^T
// block i of L z = b is
//   z_i = L_ii^-1 (b_i - sum_{k < i-1} L_ik z_k) - M_i z_{i-1}
// and block i of L^T x = z is
//   x_i = L_ii^-T (z_i - sum_{k > i+1} L_ki^T x_k) - P_i x_{i+1},
// so between a neighbour's result and this block's lies one 64 x 64 product; the
// rest is done while the neighbour is being solved, with this block's operands
// loaded before any wait.  CTA b owns blocks b, b + grid, ... in solve order and all
// CTAs are resident (cooperative launch), so the lowest unsolved block always has
// its inputs and every wait ends.  A wait is still bounded: after kFlagWaitLimit
// polls, or once another CTA has given up, the thread sets bit 2 of *err, the
// entries it still lacks read as zero, and the launch runs to its end.

constexpr int kFlagWaitLimit = 1 << 21;
constexpr unsigned long long kUnsolved = 0x7FF0DEADBEEFCAFEull;  // a signalling NaN

__device__ __forceinline__ double ld_relaxed_f64(const double *p)
{
    double v;
    asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_relaxed_s32(const int *p)
{
    int v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ bool is_unsolved(double v)
{
    return (unsigned long long)__double_as_longlong(v) == kUnsolved;
}

// Arithmetic never returns the sentinel's payload; a NaN that somehow carries it is
// stored as the canonical NaN so that it still reads as solved.
__device__ __forceinline__ void st_solved(double *p, double v)
{
    if (is_unsolved(v)) v = __longlong_as_double(0x7FFFFFFFFFFFFFFFll);
    asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}

// z[c] = v[4c] for 4c < count (c < 16; the rest are zero), once none is unsolved.
__device__ __forceinline__ void read_solved16(const double *v, int count, double (&z)[16],
                                              int *err, volatile int *abort)
{
    for (int it = 0;; ++it) {
        bool ok = true;
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            z[c] = 4 * c < count ? ld_relaxed_f64(v + 4 * c) : 0.0;
            ok &= !is_unsolved(z[c]);
        }
        if (ok) return;
        bool give_up = *abort != 0 || it >= kFlagWaitLimit;
        if (!give_up && (it & 1023) == 1023) give_up = (ld_relaxed_s32(err) & 2) != 0;
        if (give_up) {
            *abort = 1;
            atomicOr(err, 2);
#pragma unroll
            for (int c = 0; c < 16; ++c)
                if (is_unsolved(z[c])) z[c] = 0.0;
            return;
        }
        __nanosleep(32);
    }
}

// Self-test: polls solved entries that nothing writes, so every wait runs out.
__global__ void wait_timeout_selftest_kernel(const double *v, int *err)
{
    __shared__ int abort_flag;
    if (threadIdx.x == 0) abort_flag = 0;
    __syncthreads();
    double z[16];
    const int q = threadIdx.x & 3;
    read_solved16(v + q, NB - q, z, err, &abort_flag);
}

__global__ void fill_unsolved_kernel(double *__restrict__ v, int count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) v[i] = __longlong_as_double((long long)kUnsolved);
}

// The couplings M_i (i >= 1) and P_i (i < last) of the solves above, 64 x 64
// row-major each, one CTA per block; rows of L beyond n read as zero (the diagonal
// inverse of a short last block is padded with the identity).
__global__ void __launch_bounds__(256)
trsv_couple_kernel(const double *__restrict__ A, int64_t lda, int n,
                   const double *__restrict__ Linv, double *__restrict__ M,
                   double *__restrict__ P)
{
    __shared__ double T[NB][NB + 1];
    const int i = blockIdx.x, i0 = i * NB, nblk = (n + NB - 1) / NB;
    const int tid = threadIdx.x, r = tid >> 2, q = tid & 3;
    const double *Li = Linv + (int64_t)i * NB * NB;
    if (i > 0) {
        // M_i[r][c] = sum_{u <= r} Linv_i[r][u] L_i,i-1[u][c]
        const int nb = min(NB, n - i0);
        for (int e = tid; e < NB * NB; e += blockDim.x) {
            const int u = e >> 6, c = e & 63;
            T[u][c] = u < nb ? A[(int64_t)(i0 + u) * lda + (i0 - NB + c)] : 0.0;
        }
        __syncthreads();
        double acc[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) acc[c] = 0.0;
        for (int u = 0; u <= r; ++u) {
            const double l = Li[r * NB + u];
#pragma unroll
            for (int c = 0; c < 16; ++c) acc[c] = fma(l, T[u][q + 4 * c], acc[c]);
        }
        double *dst = M + (int64_t)i * NB * NB + r * NB + q;
#pragma unroll
        for (int c = 0; c < 16; ++c) dst[4 * c] = acc[c];
        __syncthreads();
    }
    if (i + 1 < nblk) {
        // P_i[t][c] = sum_{u >= t} Linv_i[u][t] L_i+1,i[c][u]
        const int nb1 = min(NB, n - i0 - NB), t = r;
        for (int e = tid; e < NB * NB; e += blockDim.x) {
            const int c = e >> 6, u = e & 63;
            T[c][u] = c < nb1 ? A[(int64_t)(i0 + NB + c) * lda + (i0 + u)] : 0.0;
        }
        __syncthreads();
        double acc[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) acc[c] = 0.0;
        for (int u = t; u < NB; ++u) {
            const double l = Li[u * NB + t];
#pragma unroll
            for (int c = 0; c < 16; ++c) acc[c] = fma(l, T[q + 4 * c][u], acc[c]);
        }
        double *dst = P + (int64_t)i * NB * NB + t * NB + q;
#pragma unroll
        for (int c = 0; c < 16; ++c) dst[4 * c] = acc[c];
    }
}

// L z = b.  Thread (r, q) = (tid / 4, tid % 4) owns row r of a block and the
// columns q, q + 4, ..., q + 60; the four threads of a row combine by shuffles.
__global__ void __launch_bounds__(TRSV_THREADS)
trsv_fwd_solved_kernel(const double *__restrict__ A, int64_t lda, int n,
                       const double *__restrict__ Linv, const double *__restrict__ M,
                       const double *__restrict__ b, double *z, int *err)
{
    __shared__ double bb[2][NB];
    __shared__ int abort_flag;
    if (threadIdx.x == 0) abort_flag = 0;
    __syncthreads();
    const int tid = threadIdx.x, r = tid >> 2, q = tid & 3;
    const int nblk = (n + NB - 1) / NB;
    int par = 0;
    for (int i = blockIdx.x; i < nblk; i += gridDim.x, par ^= 1) {
        const int i0 = i * NB, nb = min(NB, n - i0);
        const bool live = r < nb;
        const int64_t blk = (int64_t)i * NB * NB + r * NB + q;
        double li[16], mi[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            li[c] = Linv[blk + 4 * c];
            mi[c] = i > 0 ? M[blk + 4 * c] : 0.0;
        }
        const double br = live ? b[i0 + r] : 0.0;
        const double *arow = A + (int64_t)(i0 + (live ? r : 0)) * lda + q;
        double s = 0.0;
        for (int k = 0; k + 1 < i; ++k) {  // blocks k < i - 1 are full
            double lk[16], zk[16];
#pragma unroll
            for (int c = 0; c < 16; ++c) lk[c] = live ? arow[(int64_t)k * NB + 4 * c] : 0.0;
            read_solved16(z + k * NB + q, NB - q, zk, err, &abort_flag);
#pragma unroll
            for (int c = 0; c < 16; ++c) s = fma(lk[c], zk[c], s);
        }
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (q == 0) bb[par][r] = br - s;
        __syncthreads();
        double w = 0.0;
#pragma unroll
        for (int c = 0; c < 16; ++c) w = fma(li[c], bb[par][q + 4 * c], w);
        if (i > 0) {
            double zk[16];
            read_solved16(z + (i - 1) * NB + q, NB - q, zk, err, &abort_flag);
#pragma unroll
            for (int c = 0; c < 16; ++c) w = fma(-mi[c], zk[c], w);
        }
        w += __shfl_xor_sync(0xffffffffu, w, 1);
        w += __shfl_xor_sync(0xffffffffu, w, 2);
        if (q == 0 && live) st_solved(z + i0 + r, w);
    }
}

// L^T x = z, blocks in reverse order.  Thread (t, q) owns column t of a block and the
// rows q, q + 4, ..., q + 60 of the blocks below it.  The solution goes to x and, as
// the ready signal, to xs.
__global__ void __launch_bounds__(TRSV_THREADS)
trsv_bwd_solved_kernel(const double *__restrict__ A, int64_t lda, int n,
                       const double *__restrict__ Linv, const double *__restrict__ P,
                       const double *__restrict__ z, double *xs, double *__restrict__ x,
                       int *err)
{
    __shared__ double bb[2][NB];
    __shared__ int abort_flag;
    if (threadIdx.x == 0) abort_flag = 0;
    __syncthreads();
    const int tid = threadIdx.x, t = tid >> 2, q = tid & 3;
    const int nblk = (n + NB - 1) / NB;
    int par = 0;
    for (int j = blockIdx.x; j < nblk; j += gridDim.x, par ^= 1) {
        const int i = nblk - 1 - j, i0 = i * NB, nb = min(NB, n - i0);
        const int64_t blk = (int64_t)i * NB * NB;
        double li[16], pi[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) {
            li[c] = Linv[blk + (q + 4 * c) * NB + t];
            pi[c] = i + 1 < nblk ? P[blk + t * NB + q + 4 * c] : 0.0;
        }
        const double zt = t < nb ? z[i0 + t] : 0.0;
        double s = 0.0;
        for (int k = nblk - 1; k > i + 1; --k) {  // block i is full here
            const int k0 = k * NB, cnt = min(NB, n - k0) - q;
            double lk[16], xk[16];
#pragma unroll
            for (int c = 0; c < 16; ++c)
                lk[c] = 4 * c < cnt ? A[(int64_t)(k0 + q + 4 * c) * lda + i0 + t] : 0.0;
            read_solved16(xs + k0 + q, cnt, xk, err, &abort_flag);
#pragma unroll
            for (int c = 0; c < 16; ++c) s = fma(lk[c], xk[c], s);
        }
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (q == 0) bb[par][t] = zt - s;
        __syncthreads();
        double w = 0.0;
#pragma unroll
        for (int c = 0; c < 16; ++c) w = fma(li[c], bb[par][q + 4 * c], w);
        if (i + 1 < nblk) {
            const int k0 = i0 + NB;
            double xk[16];
            read_solved16(xs + k0 + q, min(NB, n - k0) - q, xk, err, &abort_flag);
#pragma unroll
            for (int c = 0; c < 16; ++c) w = fma(-pi[c], xk[c], w);
        }
        w += __shfl_xor_sync(0xffffffffu, w, 1);
        w += __shfl_xor_sync(0xffffffffu, w, 2);
        if (q == 0 && t < nb) {
            st_solved(xs + i0 + t, w);
            x[i0 + t] = w;
        }
    }
}

// Capture-safe triangular solves with the block inverses: one launch per pair of
// 64-row blocks and direction, so no CTA ever waits for another and any number of
// them may run side by side (batched, graph-recorded solves).
//  * Launch t of L z = b covers blocks 2t and 2t+1.  CTA 0 applies the previous
//    pair z_{2t-2}, z_{2t-1} to the pair's 128 rows, solves block 2t with its
//    inverse, applies z_{2t} to block 2t+1 and solves that; CTAs 1.. apply the
//    previous pair to the rows below (a warp per row, 128 columns).
//  * Launch u of L^T x = z covers blocks hi = nblk-1-2u and hi-1.  CTA 0 applies the
//    pair above, x_{hi+1}, x_{hi+2}, to the pair's 128 entries, solves block hi with
//    the transposed inverse, applies x_hi to block hi-1 and solves that; CTAs 1..
//    apply the pair above to the entries left of the pair (four threads per entry).
// Every row and entry is updated by one fixed thread group whatever the grid, so
// the result does not depend on how many CTAs a launch has.
constexpr int STEP_THREADS = 256;

__device__ __forceinline__ void trsv_fwd_step(const double *__restrict__ A, int64_t lda, int n,
                                              const double *__restrict__ Linv,
                                              double *__restrict__ x, int t, int bid, int nctas)
{
    __shared__ double zp[2 * NB], bb[2 * NB], zs[NB];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int nblk = (n + NB - 1) / NB;
    const int b0 = 2 * t, b1 = b0 + 1, r0 = b0 * NB, pc = r0 - 2 * NB;  // the previous pair is full
    if (t > 0 && tid < 2 * NB) zp[tid] = x[pc + tid];
    __syncthreads();
    if (bid == 0) {
        // bb = the pair's rows of x less the previous pair's contribution (a thread
        // pair per row, 64 columns each)
        {
            const int rl = tid >> 1, hf = tid & 1, r = r0 + rl;
            double s = 0.0;
            if (t > 0 && r < n) {
                const double *row = A + (int64_t)r * lda + pc + hf * NB;
#pragma unroll 16
                for (int c = 0; c < NB; ++c) s = fma(row[c], zp[hf * NB + c], s);
            }
            s += __shfl_xor_sync(0xffffffffu, s, 1);
            if (hf == 0) bb[rl] = r < n ? x[r] - s : 0.0;
        }
        __syncthreads();
        const int nb0 = min(NB, n - r0);
        const double z0 = gemv64_row(Linv + (int64_t)b0 * NB * NB, NB, bb, tid, NB);
        if ((tid & 3) == 0) {
            const int rr = tid >> 2;
            zs[rr] = rr < nb0 ? z0 : 0.0;
            if (rr < nb0) x[r0 + rr] = z0;
        }
        if (b1 < nblk) {
            __syncthreads();
            const int r1 = r0 + NB, nb1 = min(NB, n - r1);  // block b0 is full here
            const double s1 = gemv64_row(A + (int64_t)r1 * lda + r0, lda, zs, tid, nb1);
            if ((tid & 3) == 0 && (tid >> 2) < nb1) bb[NB + (tid >> 2)] -= s1;
            __syncthreads();
            const double z1 = gemv64_row(Linv + (int64_t)b1 * NB * NB, NB, bb + NB, tid, NB);
            if ((tid & 3) == 0 && (tid >> 2) < nb1) x[r1 + (tid >> 2)] = z1;
        }
    } else if (t > 0) {
        constexpr int nw = STEP_THREADS / 32;
        const int tw = (nctas - 1) * nw;
        for (int r = r0 + 2 * NB + (bid - 1) * nw + warp; r < n; r += tw) {
            const double *row = A + (int64_t)r * lda + pc;
            double sum = row[lane] * zp[lane];
            sum = fma(row[lane + 32], zp[lane + 32], sum);
            sum = fma(row[lane + 64], zp[lane + 64], sum);
            sum = fma(row[lane + 96], zp[lane + 96], sum);
            for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
            if (lane == 0) x[r] -= sum;
        }
    }
}

__global__ void __launch_bounds__(STEP_THREADS)
trsv_fwd_step_kernel(const double *__restrict__ A, int64_t lda, int n,
                     const double *__restrict__ Linv, double *__restrict__ x, int t)
{
    trsv_fwd_step(A, lda, n, Linv, x, t, blockIdx.x, gridDim.x);
}

__device__ __forceinline__ void trsv_bwd_step(const double *__restrict__ A, int64_t lda, int n,
                                              const double *__restrict__ Linv,
                                              double *__restrict__ x, int u, int bid, int nctas)
{
    __shared__ double xp[2 * NB], bb[2 * NB], xs[NB];
    const int tid = threadIdx.x;
    const int nblk = (n + NB - 1) / NB;
    const int hi = nblk - 1 - 2 * u, lo = hi - 1;   // lo < 0: the pair is one block
    const int a0 = (hi + 1) * NB;                    // first row of the pair above
    const int na = max(0, min(2 * NB, n - a0));      // its rows
    const int c0 = (lo >= 0 ? lo : hi) * NB;         // first entry of this pair
    if (tid < 2 * NB) xp[tid] = tid < na ? x[a0 + tid] : 0.0;
    __syncthreads();
    if (bid == 0) {
        // bb = the pair's entries of x less the pair above's contribution (a thread
        // pair per entry, 64 rows each)
        {
            const int el = tid >> 1, hf = tid & 1, c = c0 + el;
            const int cend = hi * NB + min(NB, n - hi * NB);
            double s = 0.0;
            if (c < cend) {
                const int rb = hf * NB, rn = min(NB, na - rb);
                for (int j = 0; j < rn; ++j) s = fma(A[(int64_t)(a0 + rb + j) * lda + c], xp[rb + j], s);
            }
            s += __shfl_xor_sync(0xffffffffu, s, 1);
            if (hf == 0) bb[el] = c < cend ? x[c] - s : 0.0;
        }
        __syncthreads();
        const int t = tid >> 2, q = tid & 3;
        const int bh = lo >= 0 ? NB : 0;             // block hi's offset in bb
        const int nbh = min(NB, n - hi * NB);
        const double v = gemv64_col(Linv + (int64_t)hi * NB * NB, NB, bb + bh, tid);
        if (q == 0) {
            xs[t] = t < nbh ? v : 0.0;
            if (t < nbh) x[hi * NB + t] = v;
        }
        if (lo >= 0) {
            __syncthreads();
            // bb_lo[t] -= sum_r L[hi*64 + r][lo*64 + t] x_hi[r]
            double s = 0.0;
#pragma unroll
            for (int c = 0; c < 16; ++c) {
                const int r = q + 4 * c;
                if (r < nbh) s = fma(A[(int64_t)(hi * NB + r) * lda + lo * NB + t], xs[r], s);
            }
            s += __shfl_xor_sync(0xffffffffu, s, 1);
            s += __shfl_xor_sync(0xffffffffu, s, 2);
            if (q == 0) bb[t] -= s;
            __syncthreads();
            const double w = gemv64_col(Linv + (int64_t)lo * NB * NB, NB, bb, tid);
            if (q == 0) x[lo * NB + t] = w;
        }
    } else if (na > 0) {
        const int t = tid >> 2, q = tid & 3;
        constexpr int per = STEP_THREADS / 4;
        const int tc = (nctas - 1) * per;
        for (int e0 = (bid - 1) * per; e0 < c0; e0 += tc) {
            const int c = e0 + t;
            double s = 0.0;
            if (c < c0) {
#pragma unroll 8
                for (int j = 0; j < 32; ++j) {
                    const int r = q + 4 * j;
                    if (r < na) s = fma(A[(int64_t)(a0 + r) * lda + c], xp[r], s);
                }
            }
            s += __shfl_xor_sync(0xffffffffu, s, 1);
            s += __shfl_xor_sync(0xffffffffu, s, 2);
            if (q == 0 && c < c0) x[c] -= s;
        }
    }
}

__global__ void __launch_bounds__(STEP_THREADS)
trsv_bwd_step_kernel(const double *__restrict__ A, int64_t lda, int n,
                     const double *__restrict__ Linv, double *__restrict__ x, int u)
{
    trsv_bwd_step(A, lda, n, Linv, x, u, blockIdx.x, gridDim.x);
}

// CTAs beside CTA 0 in launch t of L z = b: 32 rows below the pair each (a warp
// per row); in launch u of L^T x = z: 64 entries left of the pair each.
inline int trsv_fwd_extra(int n, int t, int64_t cap)
{
    const int below = n - (2 * t + 2) * NB;
    return (t > 0 && below > 0) ? (int)std::min<int64_t>((below + 31) / 32, cap) : 0;
}

inline int trsv_bwd_extra(int n, int u, int64_t cap)
{
    const int nblk = (n + NB - 1) / NB, lo = nblk - 2 - 2 * u;
    return (u > 0 && lo > 0) ? (int)std::min<int64_t>(((int64_t)lo * NB + 63) / 64, cap) : 0;
}

// Both triangular solves in one CTA, with the block inverses: no waiting between
// CTAs (used for matrices of one or two blocks, where one launch is cheapest).
constexpr int TRSV1_THREADS = 512;

__global__ void __launch_bounds__(TRSV1_THREADS)
trsv_single_cta_kernel(const double *__restrict__ A, int64_t lda, int n,
                       const double *__restrict__ Linv, double *__restrict__ x)
{
    __shared__ double xb[NB];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int nw = TRSV1_THREADS / 32;
    const int nblk = (n + NB - 1) / NB;
    for (int kb = 0; kb < nblk; ++kb) {  // L z = b
        const int k0 = kb * NB, nb = min(NB, n - k0);
        if (tid < NB) xb[tid] = tid < nb ? x[k0 + tid] : 0.0;
        __syncthreads();
        if (tid < 256) {
            const double z = gemv64_row(Linv + (int64_t)kb * NB * NB, NB, xb, tid, NB);
            if ((tid & 3) == 0 && (tid >> 2) < nb) x[k0 + (tid >> 2)] = z;
        }
        __syncthreads();
        if (tid < NB) xb[tid] = tid < nb ? x[k0 + tid] : 0.0;
        __syncthreads();
        if (nb == NB)
            for (int r = k0 + NB + warp; r < n; r += nw) {
                const double *row = A + (int64_t)r * lda + k0;
                double sum = fma(row[lane], xb[lane], row[lane + 32] * xb[lane + 32]);
                for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
                if (lane == 0) x[r] -= sum;
            }
        __syncthreads();
    }
    for (int kb = nblk - 1; kb >= 0; --kb) {  // L^T x = z
        const int k0 = kb * NB, nb = min(NB, n - k0);
        if (tid < NB) xb[tid] = tid < nb ? x[k0 + tid] : 0.0;
        __syncthreads();
        if (tid < 256) {
            const double v = gemv64_col(Linv + (int64_t)kb * NB * NB, NB, xb, tid);
            if ((tid & 3) == 0 && (tid >> 2) < nb) x[k0 + (tid >> 2)] = v;
        }
        __syncthreads();
        if (tid < NB) xb[tid] = tid < nb ? x[k0 + tid] : 0.0;
        __syncthreads();
        for (int t = tid; t < k0; t += TRSV1_THREADS) {
            double sum = 0.0;
            for (int r = 0; r < nb; ++r) sum = fma(A[(int64_t)(k0 + r) * lda + t], xb[r], sum);
            x[t] -= sum;
        }
        __syncthreads();
    }
}

// Cooperative kernels of this process run one at a time on the device: each one
// waits for the previous one (an event chain across streams), so two grids that
// each need every SM are never resident together.
int launch_cooperative(const void *fn, int grid, int threads, void **args, cudaStream_t s)
{
    static std::mutex mu;
    static cudaEvent_t last[64] = {};
    static bool recorded[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    if (dev < 0 || dev >= 64) return QMLG_E_ARG;
    std::lock_guard<std::mutex> lock(mu);
    if (last[dev] == nullptr) {
        e = cudaEventCreateWithFlags(&last[dev], cudaEventDisableTiming);
        if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    }
    if (recorded[dev]) {
        e = cudaStreamWaitEvent(s, last[dev], 0);
        if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    }
    e = cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(threads), args, 0, s);
    qmlg::count_launches(1);
    if (e == cudaSuccess) e = cudaEventRecord(last[dev], s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    recorded[dev] = true;
    return QMLG_OK;
}

// Cooperative kernels are off while the stream is being captured (an event
// recorded outside the capture cannot order it) and on threads that turned them
// off (qmlg_set_thread_cooperative).
bool cooperative_allowed(cudaStream_t s)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) return false;
    return cs == cudaStreamCaptureStatusNone && qmlg::cooperative_on();
}

int trsv_grid(int &grid)
{
    static int cached = 0;
    static std::once_flag once;
    static int status = QMLG_OK;
    std::call_once(once, [] {
        int dev = 0, sms = 0, per_sm = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, trsv_fwd_coop_kernel,
                                                              TRSV_THREADS, 0);
        int per_sm2 = 0, per_sm3 = 0, per_sm4 = 0;
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, trsv_bwd_coop_kernel,
                                                              TRSV_THREADS, 0);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm3, trsv_fwd_solved_kernel,
                                                              TRSV_THREADS, 0);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm4, trsv_bwd_solved_kernel,
                                                              TRSV_THREADS, 0);
        if (e != cudaSuccess) {
            status = qmlg::set_cuda_error(e);
            return;
        }
        // one CTA per SM: enough for the memory-bound updates, cheaper grid barriers
        cached = std::min(std::min(per_sm, per_sm2), std::min(per_sm3, per_sm4)) >= 1 ? sms : 0;
        if (cached < 2) status = QMLG_E_CUDA;
    });
    grid = cached;
    return status;
}

__global__ void or_flag_kernel(int *__restrict__ dst, const int *__restrict__ src)
{
    if (*src != 0) atomicOr(dst, *src);
}

__global__ void fill_nan_kernel(double *__restrict__ x, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = nan("");
}

}  // namespace

// ===================================================================== API ==

namespace qmlg {

int cholesky_fp64(double *A, int n, int64_t lda, double shift, int *d_info, cudaStream_t s,
                  int npiv, bool coupled)
{
    // npiv < n (a multiple of 64): only the first npiv pivots; the trailing
    // (n - npiv) block is left holding its Schur complement
    const int np = (npiv < 0 || npiv > n) ? n : npiv;
    for (int k0 = 0; k0 < np; k0 += NB) {
        // coupled: the rows from np + k0 + NB on are zero in this panel (their pivot
        // has not come), so the panel solve and the trailing update stop there; the
        // kernels take the row bound as their n
        const int ne = coupled ? std::min(n, np + k0 + NB) : n;
        { potrf_diag_kernel<<<1, 256, 0, s>>>(A, lda, ne, k0, shift, d_info); qmlg::count_launches(1); }
        const int below = ne - (k0 + NB);
        if (below > 0) {
            const int st = launch_trsm(A, lda, ne, k0, d_info, 0, 0, 0, nullptr, nullptr, s);
            if (st != QMLG_OK) return st;
            const int64_t t = ceil_div(below, 64);
            { syrk_update_kernel<<<(unsigned)(t * (t + 1) / 2), 256, 0, s>>>(A, lda, ne, k0, d_info); qmlg::count_launches(1); }
        }
    }
    return check_launch();
}

int potrs_fp64(const double *A, int n, int64_t lda, double *x, cudaStream_t s)
{
    int grid = 0;
    int st = trsv_grid(grid);
    if (st != QMLG_OK) return st;
    grid = std::max(2, sm_limit(grid));
    if (!cooperative_allowed(s)) return QMLG_E_ARG;  // the plain FP64 solve is not capture-safe
    void *args[] = {(void *)&A, (void *)&lda, (void *)&n, (void *)&x};
    st = launch_cooperative((const void *)trsv_fwd_coop_kernel, grid, TRSV_THREADS, args, s);
    if (st == QMLG_OK)
        st = launch_cooperative((const void *)trsv_bwd_coop_kernel, grid, TRSV_THREADS, args, s);
    return st;
}

// R[i][j] <- R[j][i] for j < i, R[i][i] <- diag[i]: restores the lower triangle from
// the untouched upper one before an FP64 refactorisation.
__global__ void mirror_kernel(double *__restrict__ A, int64_t lda, int n,
                              const double *__restrict__ diag)
{
    __shared__ double T[32][33];
    const int bi = blockIdx.y, bj = blockIdx.x;  // tile (rows bi, cols bj), bj <= bi
    if (bj > bi) return;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int k = ty; k < 32; k += 8) {
        const int r = bj * 32 + k, c = bi * 32 + tx;  // source R[r][c], r <= c
        T[k][tx] = (r < n && c < n) ? A[(int64_t)r * lda + c] : 0.0;
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
        const int i = bi * 32 + k, j = bj * 32 + tx;  // dest R[i][j] = R[j][i]
        if (i < n && j < n && j <= i) A[(int64_t)i * lda + j] = (i == j) ? diag[i] : T[tx][k];
    }
}

int mirror_upper_to_lower(double *A, int n, int64_t lda, const double *diag, cudaStream_t s)
{
    const int t = (int)ceil_div(n, 32);
    { mirror_kernel<<<dim3(t, t), dim3(32, 8), 0, s>>>(A, lda, n, diag); qmlg::count_launches(1); }
    return check_launch();
}

// Two-level emulated-FP64 factorisation.  Outer panels of NBO = 512 columns: inside
// a panel, 64-column steps (FP64 diagonal block and TRSM, emulated update of the
// panel's remaining columns with K = 64); after the panel, one emulated rank-512
// update of the whole trailing matrix (K = 512, exact levels, one FP64 epilogue per
// element).
constexpr int NBO = 512;

size_t emulated_factor_ws(int n)
{
    const size_t rpad = (size_t)ceil_div(n < 1 ? 1 : n, 128) * 128;
    WorkspacePlan p;
    p.add<__nv_bfloat16>((size_t)kEmuMaxSlices * rpad * NBO);  // outer panel digits
    p.add<int>(rpad);
    p.add<__nv_bfloat16>((size_t)kEmuMaxSlices * rpad * NB);   // inner block digits
    p.add<int>(rpad);
    p.add<int>(4);                                             // device error flag
    p.add<double>((size_t)ceil_div(n < 1 ? 1 : n, NB) * NB * NB);  // diagonal-block inverses
    p.add<double>((size_t)2 * ceil_div(n < 1 ? 1 : n, NB) * NB * NB);  // block couplings
    p.add<double>((size_t)2 * ceil_div(n < 1 ? 1 : n, NB) * NB);       // solved entries
    return p.total();
}

// Internal second stream and events of the calling thread on the current device,
// created on first use (the look-ahead below forks onto it and joins back).
struct AuxStream {
    cudaStream_t stream = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};

int aux_stream(AuxStream *&out)
{
    thread_local AuxStream pool[16];
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_cuda_error(e);
    if (dev < 0 || dev >= 16) return QMLG_E_ARG;
    AuxStream &a = pool[dev];
    if (a.stream == nullptr) {
        e = cudaStreamCreateWithFlags(&a.stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&a.fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&a.join, cudaEventDisableTiming);
        if (e != cudaSuccess) return set_cuda_error(e);
    }
    out = &a;
    return QMLG_OK;
}

// The 64-wide steps of one 512-column panel [K0, K1): FP64 diagonal block and
// TRSM, then the emulated K = 64 update of the panel's remaining columns.
int factor_panel(double *A, int n, int64_t lda, double shift, int K0, int K1, int rpad,
                 int slices, __nv_bfloat16 *dig_in, int *exp_in, int *d_info, int *d_err,
                 cudaStream_t s, int update_ctas)
{
    for (int k0 = K0; k0 < K1; k0 += NB) {
        { potrf_diag_kernel<<<1, 256, 0, s>>>(A, lda, n, k0, shift, d_info); count_launches(1); }
        const int r1 = k0 + NB;
        if (r1 >= n) break;
        // the solved rows' digit planes feed the panel's own K = 64 update
        const bool inner = r1 < K1;
        const int drows = inner ? std::min(rpad, (int)ceil_div(n - r1, 128) * 128) : 0;
        int st = launch_trsm(A, lda, n, k0, d_info, slices, rpad, drows, inner ? dig_in : nullptr,
                             inner ? exp_in : nullptr, s);
        if (st != QMLG_OK) return st;
        if (inner) {
            st = emu_tc_update(A, lda, r1, K1, r1, n, dig_in, exp_in, NB, rpad, slices, 0, 0, 1,
                               d_err, s, update_ctas);
            if (st != QMLG_OK) return st;
        }
    }
    return check_launch();
}

// SMs kept free for the panel chain while the rest of the trailing matrix, of order
// m, is updated beside it.  The update's work grows as m^2 and the chain's as m, so
// the share grows as m falls: 12, 24 then 40 of 152 SMs.  The bands come from
// per-step timings at N = 20000 and 40000 with fixed reserves of 4 to 64 SMs, then
// whole factorisations: 12/24/40 took 639.0 ms at N = 40000 against 641.6 ms for
// 16/32/48, 646.8 ms for 20/36/52 and 640.0 ms for five finer bands.
inline int chain_reserve(int sms, int m)
{
    const int per152 = m >= 30000 ? 12 : (m >= 17000 ? 24 : 40);
    return std::max(1, per152 * sms / 152);
}

// Look-ahead schedule.  After panel p is factorised its rank-512 update is split:
// (1) the next panel's columns [K1, K2) on the caller's stream; then (2) all
// columns right of K2 on the caller's stream with a grid that leaves a few SMs
// free, while the next panel's 64-wide FP64 chain runs on the auxiliary stream in
// those SMs.  The two touch disjoint columns; the next outer step joins them.
int emulated_factor(double *A, int n, int64_t lda, double shift, Workspace &ws, int *d_info,
                    EmulatedFactor &f, cudaStream_t s, int slices, int npiv, bool coupled)
{
    // npiv < n (a multiple of 64): only the first npiv pivots; the trailing
    // (n - npiv) block is left holding its Schur complement
    const int np = (npiv < 0 || npiv > n) ? n : npiv;
    // coupled ([[A_p, E], [E^T, 0]], as cholesky_fp64): the rows live once the
    // pivots before c are taken end at np + c; the launches stop there
    auto live_end = [&](int c) { return coupled ? std::min(n, np + c) : n; };
    const int rpad = (int)ceil_div(n, 128) * 128;
    __nv_bfloat16 *dig_out = ws.take<__nv_bfloat16>((size_t)kEmuMaxSlices * rpad * NBO);
    int *exp_out = ws.take<int>((size_t)rpad);
    __nv_bfloat16 *dig_in = ws.take<__nv_bfloat16>((size_t)kEmuMaxSlices * rpad * NB);
    int *exp_in = ws.take<int>((size_t)rpad);
    int *d_err = ws.take<int>(4);
    double *linv = ws.take<double>((size_t)ceil_div(n, NB) * NB * NB);
    double *couple = ws.take<double>((size_t)2 * ceil_div(n, NB) * NB * NB);
    double *solved = ws.take<double>((size_t)2 * ceil_div(n, NB) * NB);
    if (dig_out == nullptr || exp_out == nullptr || dig_in == nullptr || exp_in == nullptr ||
        d_err == nullptr || linv == nullptr || couple == nullptr || solved == nullptr)
        return QMLG_E_WORKSPACE;
    cudaError_t e = cudaMemsetAsync(d_err, 0, sizeof(int), s);
    if (e != cudaSuccess) return set_cuda_error(e);
    AuxStream *aux = nullptr;
    int st = aux_stream(aux);
    if (st != QMLG_OK) return st;
    const int sms = tc_sm_count();
    // SMs left to the panel chain.  Threads that run many solves side by side
    // (cooperative kernels off, e.g. batched fits) keep one stream per solve and
    // skip the look-ahead, so concurrent solves do not share the auxiliary stream.
    const bool lookahead = sms >= 64 && cooperative_on();
    st = factor_panel(A, live_end(std::min(NBO, np)), lda, shift, 0, std::min(NBO, np), rpad, slices,
                      dig_in, exp_in, d_info, d_err, s, 0);
    for (int K0 = 0; K0 < np && st == QMLG_OK; K0 += NBO) {
        const int K1 = std::min(K0 + NBO, np);
        if (K1 >= n) break;
        const int K2 = std::min(K1 + NBO, np);  // the next panel's pivot columns [K1, K2)
        const bool more = K2 > K1;
        const int kw = K1 - K0;
        const int kp = (int)ceil_div(kw, 64) * 64;
        const int ne = live_end(K1);  // rows with a nonzero entry in this panel end here
        st = slice_rows(A, lda, K1, ne - K1, K0, kw, kp, rpad, slices, dig_out, exp_out, d_info, s);
        if (st != QMLG_OK) break;
        // (1) the next panel's columns
        if (more)
            st = emu_tc_update(A, lda, K1, K2, K1, ne, dig_out, exp_out, kp, rpad, slices, 0, 0, 1,
                               d_err, s, 0);
        if (st != QMLG_OK) break;
        if (more && K2 < ne && lookahead) {
            const int reserve = chain_reserve(sms, ne - K2);
            // fork: the next panel's chain on the auxiliary stream
            if ((e = cudaEventRecord(aux->fork, s)) != cudaSuccess ||
                (e = cudaStreamWaitEvent(aux->stream, aux->fork, 0)) != cudaSuccess) {
                st = set_cuda_error(e);
                break;
            }
            // (2) the rest of the trailing matrix, leaving `reserve` SMs free
            st = emu_tc_update(A, lda, K2, ne, K2, ne, dig_out, exp_out, kp, rpad, slices, K2 - K1,
                               K2 - K1, 1, d_err, s, sms - reserve);
            if (st == QMLG_OK)
                st = factor_panel(A, live_end(K2), lda, shift, K1, K2, rpad, slices, dig_in, exp_in,
                                  d_info, d_err, aux->stream, -1);
            // join before the next outer step reads the panel (and reuses dig_out)
            if (st == QMLG_OK && ((e = cudaEventRecord(aux->join, aux->stream)) != cudaSuccess ||
                                  (e = cudaStreamWaitEvent(s, aux->join, 0)) != cudaSuccess))
                st = set_cuda_error(e);
        } else {
            if (K2 < ne)
                st = emu_tc_update(A, lda, K2, ne, K2, ne, dig_out, exp_out, kp, rpad, slices, K2 - K1,
                                   K2 - K1, 1, d_err, s, 0);
            if (st == QMLG_OK && more)
                st = factor_panel(A, live_end(K2), lda, shift, K1, K2, rpad, slices, dig_in, exp_in,
                                  d_info, d_err, s, 0);
        }
    }
    if (st != QMLG_OK) return st;
    const unsigned nblk = (unsigned)ceil_div(n, NB);
    if (np == n) {
        invert_diag_blocks_kernel<<<nblk, 64, 0, s>>>(A, lda, n, linv);
        trsv_couple_kernel<<<nblk, 256, 0, s>>>(A, lda, n, linv, couple,
                                                couple + (size_t)nblk * NB * NB);
        count_launches(2);
    }
    f.A = A;
    f.n = n;
    f.lda = lda;
    f.slices = slices;
    f.d_err = d_err;
    f.Linv = linv;
    f.M = couple;
    f.P = couple + (size_t)nblk * NB * NB;
    f.solved = solved;
    return check_launch();
}

// QMLG_E_TIMEOUT if a bounded tensor-core wait gave up (the flag is set on device).
int read_device_flag(const int *d_flag, cudaStream_t s)
{
    int h = 0;
    const int st = read_back(&h, d_flag, sizeof(int), s);
    if (st != QMLG_OK) return st;
    return h != 0 ? QMLG_E_TIMEOUT : QMLG_OK;
}

int emulated_potrs(const EmulatedFactor &f, double *x, cudaStream_t s)
{
    if (f.Linv == nullptr) return potrs_fp64(f.A, f.n, f.lda, x, s);
    int grid = 0;
    int st = trsv_grid(grid);
    if (st != QMLG_OK) return st;
    grid = std::max(2, sm_limit(grid));
    const double *A = f.A, *Linv = f.Linv;
    int64_t lda = f.lda;
    int n = f.n;
    if (!cooperative_allowed(s)) {
        const int nblk = (int)ceil_div(n, NB);
        if (nblk <= 2) {
            { trsv_single_cta_kernel<<<1, TRSV1_THREADS, 0, s>>>(A, lda, n, Linv, x); count_launches(1); }
            return check_launch();
        }
        const int64_t cap = 4 * (int64_t)std::max(1, tc_sm_count());
        const int steps = (nblk + 1) / 2;
        for (int t = 0; t < steps; ++t)
            trsv_fwd_step_kernel<<<1 + trsv_fwd_extra(n, t, cap), STEP_THREADS, 0, s>>>(A, lda, n, Linv, x, t);
        for (int u = 0; u < steps; ++u)
            trsv_bwd_step_kernel<<<1 + trsv_bwd_extra(n, u, cap), STEP_THREADS, 0, s>>>(A, lda, n, Linv, x, u);
        count_launches(2 * steps);
        return check_launch();
    }
    const int nblk = (int)ceil_div(n, NB), count = 2 * nblk * NB;
    { fill_unsolved_kernel<<<(unsigned)ceil_div(count, 256), 256, 0, s>>>(f.solved, count); count_launches(1); }
    const double *M = f.M, *P = f.P, *zc = f.solved;
    double *z = f.solved, *xs = f.solved + (size_t)nblk * NB;
    int *err = f.d_err;
    void *fa[] = {(void *)&A, (void *)&lda, (void *)&n, (void *)&Linv, (void *)&M,
                  (void *)&x, (void *)&z, (void *)&err};
    void *ba[] = {(void *)&A, (void *)&lda, (void *)&n, (void *)&Linv, (void *)&P,
                  (void *)&zc, (void *)&xs, (void *)&x, (void *)&err};
    st = launch_cooperative((const void *)trsv_fwd_solved_kernel, grid, TRSV_THREADS, fa, s);
    if (st == QMLG_OK)
        st = launch_cooperative((const void *)trsv_bwd_solved_kernel, grid, TRSV_THREADS, ba, s);
    return st;
}

size_t residual_ws(int n)
{
    WorkspacePlan p;
    p.add<AccPart>((size_t)ceil_div(n, RES_CHUNK) * (size_t)n);
    return p.total();
}

int residual_dd(const double *A, int n, int64_t lda, const double *diag, double lambda,
                const double *x, const double *y, double *r, Workspace &ws, cudaStream_t s)
{
    const int nchunks = (int)ceil_div(n, RES_CHUNK);
    AccPart *partial = ws.take<AccPart>((size_t)nchunks * n);
    if (partial == nullptr) return QMLG_E_WORKSPACE;
    static std::once_flag once;
    static int attr = QMLG_OK;
    std::call_once(once, [] { attr = res_smem_attr(symv_exact_partial_kernel); });
    if (attr != QMLG_OK) return attr;
    { symv_exact_partial_kernel<<<dim3((unsigned)ceil_div(n, RES_ROWS), nchunks), 256, RES_SMEM, s>>>(
        A, lda, n, diag, x, partial); qmlg::count_launches(1); }
    { residual_finish_kernel<<<(int)ceil_div(n, 256), 256, 0, s>>>(partial, nchunks, n, lambda, x,
                                                                 y, r); qmlg::count_launches(1); }
    return check_launch();
}

}  // namespace qmlg

extern "C" size_t qmlg_cholesky_workspace_size(int n)
{
    (void)n;
    qmlg::WorkspacePlan p;
    p.add<int>(4);
    return p.total();
}

extern "C" int qmlg_cholesky(double *A, int n, int64_t lda, double lambda, void *workspace,
                             size_t ws_bytes, void *stream)
{
    if (n < 0 || lda < n || (n > 0 && A == nullptr)) return QMLG_E_ARG;
    if (n == 0) return QMLG_OK;
    qmlg::Workspace ws(workspace, ws_bytes);
    int *d_info = ws.take<int>(4);
    if (d_info == nullptr) return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    cudaError_t e = cudaMemsetAsync(d_info, 0, sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    int st = qmlg::cholesky_fp64(A, n, lda, lambda, d_info, s);
    if (st != QMLG_OK) return st;
    int info = 0;
    st = qmlg::read_back(&info, d_info, sizeof(int), s);
    return st != QMLG_OK ? st : info;
}

extern "C" size_t qmlg_cholesky_mixed_workspace_size(int n)
{
    qmlg::WorkspacePlan p;
    p.add<int>(4);
    p.add<char>(qmlg::emulated_factor_ws(n));
    return p.total();
}

extern "C" int qmlg_cholesky_mixed(double *A, int n, int64_t lda, double lambda, void *workspace,
                                   size_t ws_bytes, void *stream)
{
    if (n < 0 || lda < n || (n > 0 && A == nullptr)) return QMLG_E_ARG;
    if (n == 0) return QMLG_OK;
    if (ws_bytes < qmlg_cholesky_mixed_workspace_size(n)) return QMLG_E_WORKSPACE;
    qmlg::Workspace ws(workspace, ws_bytes);
    int *d_info = ws.take<int>(4);
    cudaStream_t s = qmlg::as_stream(stream);
    cudaError_t e = cudaMemsetAsync(d_info, 0, sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    qmlg::EmulatedFactor f;
    int st = qmlg::emulated_factor(A, n, lda, lambda, ws, d_info, f, s);
    if (st != QMLG_OK) return st;
    if ((st = qmlg::read_device_flag(f.d_err, s)) != QMLG_OK) return st;
    int info = 0;
    st = qmlg::read_back(&info, d_info, sizeof(int), s);
    return st != QMLG_OK ? st : info;
}

extern "C" size_t qmlg_selftest_wait_timeout_workspace_size(void)
{
    qmlg::WorkspacePlan p;
    p.add<double>(NB);
    p.add<int>(4);
    return p.total();
}

extern "C" int qmlg_selftest_wait_timeout(void *workspace, size_t ws_bytes, void *stream)
{
    qmlg::Workspace ws(workspace, ws_bytes);
    double *v = ws.take<double>(NB);
    int *err = ws.take<int>(4);
    if (v == nullptr || err == nullptr) return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    cudaError_t e = cudaMemsetAsync(err, 0, sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    { fill_unsolved_kernel<<<1, NB, 0, s>>>(v, NB); qmlg::count_launches(1); }
    { wait_timeout_selftest_kernel<<<1, NB, 0, s>>>(v, err); qmlg::count_launches(1); }
    int st = qmlg::check_launch();
    if (st != QMLG_OK) return st;
    int h = 0;
    if ((st = qmlg::read_back(&h, err, sizeof(int), s)) != QMLG_OK) return st;
    return (h & 2) ? QMLG_E_TIMEOUT : QMLG_OK;
}

extern "C" int qmlg_cholesky_solve_factored(const double *U, int n, int64_t lda, const double *y,
                                            double *x, void *stream)
{
    if (n < 0 || lda < n || (n > 0 && (U == nullptr || y == nullptr || x == nullptr)))
        return QMLG_E_ARG;
    if (n == 0) return QMLG_OK;
    cudaStream_t s = qmlg::as_stream(stream);
    if (x != y) {
        cudaError_t e = cudaMemcpyAsync(x, y, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    }
    return qmlg::potrs_fp64(U, n, lda, x, s);
}

extern "C" size_t qmlg_residual_workspace_size(int n) { return qmlg::residual_ws(n); }

extern "C" int qmlg_residual_dd(const double *A, int n, int64_t lda, const double *diag,
                                double lambda, const double *x, const double *y, double *r,
                                void *workspace, size_t ws_bytes, void *stream)
{
    if (n < 0 || lda < n) return QMLG_E_ARG;
    if (n == 0) return QMLG_OK;
    if (A == nullptr || diag == nullptr || x == nullptr || y == nullptr || r == nullptr)
        return QMLG_E_ARG;
    qmlg::Workspace ws(workspace, ws_bytes);
    return qmlg::residual_dd(A, n, lda, diag, lambda, x, y, r, ws, qmlg::as_stream(stream));
}

// ------------------------------------------------------------ full solve --

extern "C" size_t qmlg_solve_workspace_size(int n, int precision)
{
    qmlg::WorkspacePlan p;
    p.add<int>(4);                       // info
    p.add<double>(4);                    // norm sums
    p.add<double>((size_t)n);            // saved diagonal
    p.add<double>((size_t)n);            // residual / correction
    p.add<char>(qmlg::residual_ws(n));   // residual partials
    if (precision == QMLG_PREC_MIXED) p.add<char>(qmlg::emulated_factor_ws(n));
    return p.total();
}

namespace {

struct SolveCtx {
    double *A;
    int n;
    int64_t lda;
    const double *y;
    double *x;
    double lambda;
    int *d_info;
    double *d_sums;
    double *diag;
    double *r;
    qmlg::Workspace *ws;
    size_t ws_mark;
    cudaStream_t s;
};

int read_info(SolveCtx &c, int &info)
{
    return qmlg::read_back(&info, c.d_info, sizeof(int), c.s);
}

// Iterative refinement: r = y - (A + lambda I) x summed exactly, dx = solve(r),
// x += dx, until |dx|/|x| <= tol or the correction stops shrinking.
template <class SolveFn>
int refine(SolveCtx &c, const QmlgRefineOpts &o, SolveFn solve_fn, QmlgSolveReport &rep,
           bool &stalled)
{
    stalled = false;
    double prev = INFINITY;
    rep.last_correction = INFINITY;
    for (int it = 0; it < o.max_outer; ++it) {
        c.ws->used = c.ws_mark;
        int st = qmlg::residual_dd(c.A, c.n, c.lda, c.diag, c.lambda, c.x, c.y, c.r, *c.ws, c.s);
        if (st != QMLG_OK) return st;
        st = solve_fn(c.r);
        if (st != QMLG_OK) return st;
        cudaError_t e = cudaMemsetAsync(c.d_sums, 0, 2 * sizeof(double), c.s);
        if (e != cudaSuccess) return qmlg::set_cuda_error(e);
        { axpy_norms_kernel<<<(int)qmlg::ceil_div(c.n, 256), 256, 0, c.s>>>(c.x, c.r, c.n, c.d_sums); qmlg::count_launches(1); }
        double h[2];
        st = qmlg::read_back(h, c.d_sums, sizeof(h), c.s);
        if (st != QMLG_OK) return st;
        const double rel = std::sqrt(h[0]) / std::fmax(std::sqrt(h[1]), 1e-300);
        rep.outer_iterations = it + 1;
        rep.last_correction = rel;
        if (!(rel == rel)) {
            stalled = true;
            return QMLG_OK;
        }
        if (rel <= o.tol) return QMLG_OK;
        // linear convergence: the next correction is about rel * (rel / prev)
        if (prev < INFINITY && rel * (rel / prev) <= 0.1 * o.tol) return QMLG_OK;
        if (rel > 0.5 * prev) {
            stalled = true;
            return QMLG_OK;
        }
        prev = rel;
    }
    stalled = rep.last_correction > o.tol;
    return QMLG_OK;
}

}  // namespace

extern "C" int qmlg_solve(double *A, int n, int64_t lda, const double *y, double *x,
                          double lambda, int precision, const QmlgRefineOpts *opts,
                          QmlgSolveReport *report, void *workspace, size_t ws_bytes, void *stream)
{
    if (n < 0 || lda < n) return QMLG_E_ARG;
    if (precision != QMLG_PREC_FP64 && precision != QMLG_PREC_MIXED) return QMLG_E_ARG;
    QmlgSolveReport rep{};
    rep.precision_used = precision;
    if (n == 0) {
        if (report) *report = rep;
        return QMLG_OK;
    }
    if (A == nullptr || y == nullptr || x == nullptr) return QMLG_E_ARG;
    if (ws_bytes < qmlg_solve_workspace_size(n, precision)) return QMLG_E_WORKSPACE;
    QmlgRefineOpts o{10, 50, 1e-15, 0.0, 1, 0};
    if (opts) o = *opts;
    const int slices = o.slices == 0 ? qmlg::kEmuMaxSlices : o.slices;
    if (slices < 4 || slices > qmlg::kEmuMaxSlices) return QMLG_E_ARG;

    cudaStream_t s = qmlg::as_stream(stream);
    qmlg::Workspace ws(workspace, ws_bytes);
    SolveCtx c{A, n, lda, y, x, lambda, ws.take<int>(4), ws.take<double>(4),
               ws.take<double>((size_t)n), ws.take<double>((size_t)n), &ws, 0, s};
    c.ws_mark = ws.used;
    cudaError_t e = cudaMemsetAsync(c.d_info, 0, sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    { copy_diag_kernel<<<(int)qmlg::ceil_div(n, 256), 256, 0, s>>>(A, lda, n, c.diag); qmlg::count_launches(1); }

    int st = QMLG_OK, info = 0;
    bool stalled = false;
    if (precision == QMLG_PREC_MIXED) {
        // Emulated-FP64 factor on the tensor cores, in place like the FP64 one.
        qmlg::EmulatedFactor f;
        st = qmlg::emulated_factor(A, n, lda, lambda, ws, c.d_info, f, s, slices);
        if (st != QMLG_OK) return st;
        if ((st = read_info(c, info)) != QMLG_OK) return st;
        if ((st = qmlg::read_device_flag(f.d_err, s)) != QMLG_OK) return st;
        rep.info = info;
        if (info == 0) {
            e = cudaMemcpyAsync(x, y, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s);
            if (e != cudaSuccess) return qmlg::set_cuda_error(e);
            if ((st = qmlg::emulated_potrs(f, x, s)) != QMLG_OK) return st;
            c.ws_mark = ws.used;
            st = refine(c, o, [&](double *v) { return qmlg::emulated_potrs(f, v, s); }, rep, stalled);
            if (st != QMLG_OK) return st;
            if ((st = qmlg::read_device_flag(f.d_err, s)) != QMLG_OK) return st;
        }
        if ((info != 0 || stalled) && o.allow_fallback) {
            rep.fell_back = 1;
            precision = QMLG_PREC_FP64;
            e = cudaMemsetAsync(c.d_info, 0, sizeof(int), s);
            if (e != cudaSuccess) return qmlg::set_cuda_error(e);
            if ((st = qmlg::mirror_upper_to_lower(A, n, lda, c.diag, s)) != QMLG_OK) return st;
        } else {
            rep.backward_error = 0.0;
            if (report) *report = rep;
            if (info != 0) return info;
            return stalled ? QMLG_E_NOT_CONVERGED : QMLG_OK;
        }
    }

    // Plain FP64: factor A in place (upper triangle, like dpotrf("U")).
    rep.precision_used = QMLG_PREC_FP64;
    if ((st = qmlg::cholesky_fp64(A, n, lda, lambda, c.d_info, s)) != QMLG_OK) return st;
    if ((st = read_info(c, info)) != QMLG_OK) return st;
    rep.info = info;
    if (info != 0) {
        { fill_nan_kernel<<<(int)qmlg::ceil_div(n, 256), 256, 0, s>>>(x, n); qmlg::count_launches(1); }
        if (report) *report = rep;
        return info;
    }
    e = cudaMemcpyAsync(x, y, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    if ((st = qmlg::potrs_fp64(A, n, lda, x, s)) != QMLG_OK) return st;
    if (o.max_outer > 0) {
        st = refine(c, o, [&](double *v) { return qmlg::potrs_fp64(A, n, lda, v, s); }, rep,
                    stalled);
        if (st != QMLG_OK) return st;
    }
    if (report) *report = rep;
    e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    return (o.max_outer > 0 && stalled) ? QMLG_E_NOT_CONVERGED : QMLG_OK;
}

// ------------------------------------------------- capture-safe mixed solve --

extern "C" size_t qmlg_solve_async_workspace_size(int n)
{
    return qmlg_solve_workspace_size(n, QMLG_PREC_MIXED);
}

extern "C" int qmlg_solve_async(double *A, int n, int64_t lda, const double *y, double *x,
                                double lambda, int refine_steps, int *d_status,
                                double *d_correction, void *workspace, size_t ws_bytes,
                                void *stream)
{
    if (n < 0 || lda < n || refine_steps < 0 || d_status == nullptr) return QMLG_E_ARG;
    if (n == 0) return QMLG_OK;
    if (A == nullptr || y == nullptr || x == nullptr) return QMLG_E_ARG;
    if (ws_bytes < qmlg_solve_async_workspace_size(n)) return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    qmlg::Workspace ws(workspace, ws_bytes);
    ws.take<int>(4);  // same layout as qmlg_solve; status lives in d_status here
    double *d_sums = ws.take<double>(4);
    double *diag = ws.take<double>((size_t)n);
    double *r = ws.take<double>((size_t)n);
    if (d_sums == nullptr || diag == nullptr || r == nullptr) return QMLG_E_WORKSPACE;
    const size_t mark = ws.used;
    cudaError_t e = cudaMemsetAsync(d_status, 0, 2 * sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    { copy_diag_kernel<<<(int)qmlg::ceil_div(n, 256), 256, 0, s>>>(A, lda, n, diag); qmlg::count_launches(1); }
    ws.used = mark + qmlg::residual_ws(n);  // the residual partials come first
    qmlg::EmulatedFactor f;
    int st = qmlg::emulated_factor(A, n, lda, lambda, ws, d_status, f, s);
    if (st != QMLG_OK) return st;
    e = cudaMemcpyAsync(x, y, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    if ((st = qmlg::emulated_potrs(f, x, s)) != QMLG_OK) return st;
    for (int it = 0; it < refine_steps; ++it) {
        qmlg::Workspace rws(workspace, ws_bytes);
        rws.used = mark;
        if ((st = qmlg::residual_dd(A, n, lda, diag, lambda, x, y, r, rws, s)) != QMLG_OK) return st;
        if ((st = qmlg::emulated_potrs(f, r, s)) != QMLG_OK) return st;
        e = cudaMemsetAsync(d_sums, 0, 2 * sizeof(double), s);
        if (e != cudaSuccess) return qmlg::set_cuda_error(e);
        { axpy_norms_kernel<<<(int)qmlg::ceil_div(n, 256), 256, 0, s>>>(x, r, n, d_sums); qmlg::count_launches(1); }
    }
    // tensor-core and triangular-solve waits that gave up
    { or_flag_kernel<<<1, 1, 0, s>>>(d_status + 1, f.d_err); qmlg::count_launches(1); }
    if (d_correction != nullptr && refine_steps > 0) {
        e = cudaMemcpyAsync(d_correction, d_sums, 2 * sizeof(double), cudaMemcpyDeviceToDevice, s);
        if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    }
    return qmlg::check_launch();
}

namespace qmlg {

int launch_cooperative_serialised(const void *fn, int grid, int threads, void **args,
                                  cudaStream_t s)
{
    return launch_cooperative(fn, grid, threads, args, s);
}

bool cooperative_allowed_on(cudaStream_t s) { return cooperative_allowed(s); }

}  // namespace qmlg

// ------------------------------------------------------------ cho_invert --
//
// Inverse of an SPD matrix through the Schur complement of an augmented matrix:
// the first np pivots of the Cholesky factorisation of
//     M = [ A_p  E ]   (A_p = A padded with an identity to np = ceil64(n) rows,
//         [ E^T  0 ]    E = [I_n; 0], size np + n)
// give L11 = chol(A_p), L21 = E^T L11^-T and leave 0 - L21 L21^T = -A^-1 in the
// trailing n x n block.  The TRSM, the trailing updates and (mixed precision) the
// emulated tensor-core products are the factorisation's own kernels.

namespace {

// M's lower triangle (row-major view, ldm = N): A's column-major lower triangle
// (the triangle dpotrf("L") reads), identity padding, the identity coupling block.
__global__ void build_augmented_kernel(const double *__restrict__ A, int64_t lda, int n, int np,
                                       double *__restrict__ M, int64_t ldm)
{
    const int N = np + n;
    const int64_t total = (int64_t)N * N;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int r = (int)(e / N), c = (int)(e % N);
        if (c > r) continue;
        double v = 0.0;
        if (r < np) {
            if (r < n) v = A[(int64_t)r + (int64_t)c * lda];  // c <= r < n
            else v = (r == c) ? 1.0 : 0.0;
        } else if (c < np) {
            v = (c == r - np) ? 1.0 : 0.0;
        }
        M[(int64_t)r * ldm + c] = v;
    }
}

// Ainv (column-major, ldi) = -S, S the trailing block's lower triangle, mirrored.
__global__ void extract_inverse_kernel(const double *__restrict__ M, int64_t ldm, int np, int n,
                                       double *__restrict__ Ainv, int64_t ldi)
{
    const int64_t total = (int64_t)n * n;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % n), j = (int)(e / n);
        const int hi = i > j ? i : j, lo = i > j ? j : i;
        Ainv[(int64_t)i + (int64_t)j * ldi] = -M[(int64_t)(np + hi) * ldm + (np + lo)];
    }
}

}  // namespace

extern "C" size_t qmlg_cho_invert_workspace_size(int n, int precision)
{
    if (n < 1) n = 1;
    const int np = (int)qmlg::ceil_div(n, NB) * NB, N = np + n;
    qmlg::WorkspacePlan p;
    p.add<int>(4);
    p.add<double>((size_t)N * N);
    if (precision == QMLG_PREC_MIXED) p.add<char>(qmlg::emulated_factor_ws(N));
    return p.total();
}

extern "C" int qmlg_cho_invert(const double *A, int n, int64_t lda, double *Ainv, int64_t ldi,
                               int precision, void *workspace, size_t ws_bytes, void *stream)
{
    if (n < 0 || lda < n || ldi < n || (precision != QMLG_PREC_FP64 && precision != QMLG_PREC_MIXED))
        return QMLG_E_ARG;
    if (n == 0) return QMLG_OK;
    if (A == nullptr || Ainv == nullptr) return QMLG_E_ARG;
    if (ws_bytes < qmlg_cho_invert_workspace_size(n, precision)) return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    qmlg::Workspace ws(workspace, ws_bytes);
    const int np = (int)qmlg::ceil_div(n, NB) * NB, N = np + n;
    int *d_info = ws.take<int>(4);
    double *M = ws.take<double>((size_t)N * N);
    cudaError_t e = cudaMemsetAsync(d_info, 0, sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    const int blocks = (int)std::min<int64_t>(qmlg::ceil_div((int64_t)N * N, 256), 152 * 64);
    { build_augmented_kernel<<<blocks, 256, 0, s>>>(A, lda, n, np, M, N); qmlg::count_launches(1); }
    int st;
    if (precision == QMLG_PREC_MIXED) {
        qmlg::EmulatedFactor f;
        st = qmlg::emulated_factor(M, N, N, 0.0, ws, d_info, f, s, 8, np, true);
        if (st == QMLG_OK) st = qmlg::read_device_flag(f.d_err, s);
    } else {
        st = qmlg::cholesky_fp64(M, N, N, 0.0, d_info, s, np, true);
    }
    if (st != QMLG_OK) return st;
    const int eb = (int)std::min<int64_t>(qmlg::ceil_div((int64_t)n * n, 256), 152 * 64);
    { extract_inverse_kernel<<<eb, 256, 0, s>>>(M, N, np, n, Ainv, ldi); qmlg::count_launches(1); }
    int info = 0;
    st = qmlg::read_back(&info, d_info, sizeof(int), s);
    if (st != QMLG_OK) return st;
    // a pivot in the identity padding cannot fail; report A's pivot index like dpotrf
    return info > n ? n : info;
}

// ============================================================ batched fits ==
//
// qmlg_fit_batched_async: every phase of many independent fits as one grouped
// launch.  A grouped launch runs several problems' grids back to back in one grid:
// problem p owns CTAs [cta_base, cta_base + ctas) and its kernel body sees them as
// blocks 0 .. ctas-1 (the bodies above take the block index as an argument).  The
// table travels in the kernel parameter (a few KB), so the launch can be recorded
// into a graph with no host-to-device copy.

namespace {

constexpr int kMaxBatch = 128;

struct BatchEntry {
    double *A;
    int64_t lda;
    int n, k;              // k: the 64-row block this step works on
    double lambda;
    int *status;           // [0] Cholesky info, [1] flags
    double *Linv;
    double *x;
    const double *y;
    double *r;
    double *diag;
    AccPart *partial;
    double *sums;
    double *correction;
    __nv_bfloat16 *digits;  // panel solve: this problem's rows of the shared inner planes
    int *expo;
    int drows;
    int cta_base, ctas;
};

struct BatchGroup {
    int count, pad;
    BatchEntry e[kMaxBatch];
};

__device__ __forceinline__ const BatchEntry &batch_entry(const BatchGroup &g, int &local)
{
    const int bid = (int)blockIdx.x;
    int lo = 0, hi = g.count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (g.e[mid].cta_base <= bid) lo = mid;
        else hi = mid - 1;
    }
    local = bid - g.e[lo].cta_base;
    return g.e[lo];
}

__global__ void __launch_bounds__(POTRF_THREADS) potrf_group_kernel(const __grid_constant__ BatchGroup g)
{
    int b;
    const BatchEntry &e = batch_entry(g, b);
    potrf_diag_block(e.A, e.lda, e.n, e.k * NB, e.lambda, e.status);
}

__global__ void __launch_bounds__(4 * TRSM_MAX_ROWS)
trsm_group_kernel(const __grid_constant__ BatchGroup g, int slices, int rows_total)
{
    int b;
    const BatchEntry &e = batch_entry(g, b);
    trsm_panel_rows(e.A, e.lda, e.n, e.k * NB, e.status, slices, rows_total, e.drows, e.digits,
                    e.expo, b);
}

__global__ void __launch_bounds__(64) invert_group_kernel(const __grid_constant__ BatchGroup g)
{
    int b;
    const BatchEntry &e = batch_entry(g, b);
    invert_diag_block(e.A, e.lda, e.n, e.Linv, b);
}

__global__ void __launch_bounds__(STEP_THREADS) fwd_group_kernel(const __grid_constant__ BatchGroup g)
{
    int b;
    const BatchEntry &e = batch_entry(g, b);
    trsv_fwd_step(e.A, e.lda, e.n, e.Linv, e.x, e.k, b, e.ctas);
}

__global__ void __launch_bounds__(STEP_THREADS) bwd_group_kernel(const __grid_constant__ BatchGroup g)
{
    int b;
    const BatchEntry &e = batch_entry(g, b);
    trsv_bwd_step(e.A, e.lda, e.n, e.Linv, e.x, e.k, b, e.ctas);
}

__global__ void __launch_bounds__(256) symv_group_kernel(const __grid_constant__ BatchGroup g)
{
    int b;
    const BatchEntry &e = batch_entry(g, b);
    const int rb = (e.n + RES_ROWS - 1) / RES_ROWS;
    symv_exact_partial_block(e.A, e.lda, e.n, e.diag, e.x, e.partial, b % rb, b / rb);
}

__global__ void __launch_bounds__(256) finish_group_kernel(const __grid_constant__ BatchGroup g)
{
    int b;
    const BatchEntry &e = batch_entry(g, b);
    residual_finish_block(e.partial, (e.n + RES_CHUNK - 1) / RES_CHUNK, e.n, e.lambda, e.x, e.y,
                          e.r, b);
}

__global__ void __launch_bounds__(256) axpy_group_kernel(const __grid_constant__ BatchGroup g)
{
    int b;
    const BatchEntry &e = batch_entry(g, b);
    axpy_norms_block(e.x, e.r, e.n, e.sums, b);
}

enum VecOp { kCopyDiag = 0, kCopyY = 1, kZeroSums = 2, kFinishFlags = 3 };

// Small per-problem vector work: K's diagonal saved, x = y, the norm sums cleared,
// and at the end the group's wait flags ORed into every status and the last
// correction copied out.
__global__ void __launch_bounds__(256) vec_group_kernel(const __grid_constant__ BatchGroup g, int op,
                                                        const int *__restrict__ err)
{
    int b;
    const BatchEntry &e = batch_entry(g, b);
    const int i = b * 256 + (int)threadIdx.x;
    if (op == kCopyDiag) {
        if (i < e.n) e.diag[i] = e.A[(int64_t)i * e.lda + i];
    } else if (op == kCopyY) {
        if (i < e.n) e.x[i] = e.y[i];
    } else if (op == kZeroSums) {
        if (i < 2) e.sums[i] = 0.0;
    } else if (b == 0 && threadIdx.x == 0) {
        const int f = *err;
        if (f != 0) atomicOr(e.status + 1, f);
        if (e.correction != nullptr) {
            e.correction[0] = e.sums[0];
            e.correction[1] = e.sums[1];
        }
    }
}

// Host staging of one grouped launch (the table is copied into the launch).
struct BatchLauncher {
    BatchGroup g;
    int total = 0;
    void begin()
    {
        g.count = 0;
        total = 0;
    }
    BatchEntry *add(int ctas)
    {
        if (ctas <= 0 || g.count >= kMaxBatch) return nullptr;
        BatchEntry &e = g.e[g.count++];
        e = BatchEntry{};
        e.cta_base = total;
        e.ctas = ctas;
        total += ctas;
        return &e;
    }
};

// Per-fit state of a batch, carved from the workspace.
struct BatchFit {
    const QmlgBatchProblem *q;
    int n, nblk, row_k, row_p;
    double *diag, *r, *sums, *linv;
    AccPart *partial;
    void *lws;
    size_t lws_bytes;
};

struct BatchBufs {
    __nv_bfloat16 *kdig, *pdig, *idig;
    int *kexp, *pexp, *iexp, *err;
    double *knorm;
    unsigned long long *maxbuf;
    int RK, RT;
};

// The workspace layout of a batch; with base == nullptr only the size is computed.
size_t batch_carve(const QmlgBatchProblem *probs, int count, int d, char *base, BatchBufs &b,
                   std::vector<BatchFit> *fits)
{
    size_t used = 0;
    auto take = [&](size_t bytes) -> char * {
        const size_t off = qmlg::align_up(used, 256);
        used = off + bytes;
        return base != nullptr ? base + off : nullptr;
    };
    const int kp = qmlg::plane_cols(d);
    b.RK = 0;
    b.RT = 0;
    for (int p = 0; p < count; ++p) {
        if (probs[p].kind == QMLG_KIND_GAUSSIAN) b.RK += qmlg::plane_rows(probs[p].n);
        b.RT += qmlg::plane_rows(probs[p].n);
    }
    const int RK = std::max(b.RK, 128), RT = std::max(b.RT, 128);
    b.kdig = (__nv_bfloat16 *)take((size_t)qmlg::kEmuMaxSlices * RK * kp * 2);
    b.kexp = (int *)take((size_t)RK * 4);
    b.knorm = (double *)take((size_t)RK * 8);
    b.maxbuf = (unsigned long long *)take((size_t)std::max(count, 1) * 8);
    b.err = (int *)take(16);
    b.pdig = (__nv_bfloat16 *)take((size_t)qmlg::kEmuMaxSlices * RT * 512 * 2);
    b.pexp = (int *)take((size_t)RT * 4);
    b.idig = (__nv_bfloat16 *)take((size_t)qmlg::kEmuMaxSlices * RT * NB * 2);
    b.iexp = (int *)take((size_t)RT * 4);
    int rk = 0, rp = 0;
    for (int p = 0; p < count; ++p) {
        const int n = std::max(probs[p].n, 0);
        BatchFit f{};
        f.q = &probs[p];
        f.n = n;
        f.nblk = (int)qmlg::ceil_div(n, NB);
        f.row_k = probs[p].kind == QMLG_KIND_GAUSSIAN ? rk : -1;
        if (probs[p].kind == QMLG_KIND_GAUSSIAN) rk += qmlg::plane_rows(n);
        f.row_p = rp;
        rp += qmlg::plane_rows(n);
        f.diag = (double *)take((size_t)n * 8);
        f.r = (double *)take((size_t)n * 8);
        f.sums = (double *)take(16);
        f.linv = (double *)take((size_t)f.nblk * NB * NB * 8);
        f.partial = (AccPart *)take((size_t)qmlg::ceil_div(n, RES_CHUNK) * n * sizeof(AccPart));
        f.lws = nullptr;
        f.lws_bytes = 0;
        if (probs[p].kind == QMLG_KIND_LAPLACIAN) {
            f.lws_bytes = qmlg_laplacian_kernel_fixed_workspace_size(n, n, d, QMLG_KERNEL_SYMMETRIC);
            f.lws = take(f.lws_bytes);
        }
        if (fits != nullptr) fits->push_back(f);
    }
    return qmlg::align_up(used, 256) + 256;
}

}  // namespace

extern "C" size_t qmlg_fit_batched_workspace_size(const QmlgBatchProblem *problems, int count,
                                                  int d)
{
    if (problems == nullptr || count <= 0) return 256;
    BatchBufs b{};
    return batch_carve(problems, count, d, nullptr, b, nullptr);
}

extern "C" int qmlg_fit_batched_async(const QmlgBatchProblem *problems, int count, int d,
                                      int refine_steps, int tile_cols, int trsm_rows,
                                      void *workspace, size_t ws_bytes, void *stream)
{
    if (count == 0) return QMLG_OK;
    if (problems == nullptr || count < 0 || count > kMaxBatch || d < 1 || refine_steps < 0)
        return QMLG_E_ARG;
    if (tile_cols == 0) tile_cols = 64;
    if (trsm_rows == 0) trsm_rows = TRSM_MAX_ROWS;
    if ((tile_cols != 32 && tile_cols != 64) || trsm_rows < 32 || trsm_rows > TRSM_MAX_ROWS ||
        trsm_rows % 8 != 0)
        return QMLG_E_ARG;
    for (int p = 0; p < count; ++p) {
        const QmlgBatchProblem &q = problems[p];
        if (q.n < 1 || q.X == nullptr || q.ldx < d || q.y == nullptr || q.alpha == nullptr ||
            q.K == nullptr || q.status == nullptr || !(q.sigma > 0.0) || !(q.lambda >= 0.0) ||
            (q.kind != QMLG_KIND_GAUSSIAN && q.kind != QMLG_KIND_LAPLACIAN))
            return QMLG_E_ARG;
    }
    if (workspace == nullptr || ws_bytes < qmlg_fit_batched_workspace_size(problems, count, d))
        return QMLG_E_WORKSPACE;
    cudaStream_t s = qmlg::as_stream(stream);
    BatchBufs b{};
    std::vector<BatchFit> fits;
    fits.reserve((size_t)count);
    batch_carve(problems, count, d, static_cast<char *>(workspace), b, &fits);
    const int RK = std::max(b.RK, 128), RT = std::max(b.RT, 128);
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [] {
        attr = cudaFuncSetAttribute(trsm_group_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)trsm_smem(TRSM_MAX_ROWS));
        if (attr == cudaSuccess)
            attr = cudaFuncSetAttribute(symv_group_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)RES_SMEM);
    });
    if (attr != cudaSuccess) return qmlg::set_cuda_error(attr);
    static BatchLauncher L;  // 18 KB of staging, kept off the stack
    static std::mutex mu;
    std::lock_guard<std::mutex> lock(mu);
    cudaError_t e = cudaMemsetAsync(b.err, 0, sizeof(int), s);
    for (int p = 0; p < count && e == cudaSuccess; ++p)
        e = cudaMemsetAsync(problems[p].status, 0, 2 * sizeof(int), s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);

    // one grouped launch; `fill` sets a problem's entry (returns its CTA count, 0 = skip)
    auto run = [&](auto launch, auto fill) -> int {
        L.begin();
        for (BatchFit &f : fits) {
            BatchEntry tmp{};
            const int ctas = fill(f, tmp);
            if (ctas <= 0) continue;
            BatchEntry *en = L.add(ctas);
            const int base = en->cta_base;
            *en = tmp;
            en->cta_base = base;
            en->ctas = ctas;
        }
        if (L.total == 0) return QMLG_OK;
        launch(L.total);
        qmlg::count_launches(1);
        return qmlg::check_launch();
    };
    auto base_entry = [&](const BatchFit &f, BatchEntry &en) {
        en.A = f.q->K;
        en.lda = f.n;
        en.n = f.n;
        en.lambda = f.q->lambda;
        en.status = f.q->status;
        en.Linv = f.linv;
        en.y = f.q->y;
        en.r = f.r;
        en.diag = f.diag;
        en.partial = f.partial;
        en.sums = f.sums;
        en.correction = f.q->correction;
    };
    auto vec = [&](int op, auto ctas_of, double *(*xsel)(const BatchFit &)) -> int {
        return run([&](int grid) { vec_group_kernel<<<grid, 256, 0, s>>>(L.g, op, b.err); },
                   [&](const BatchFit &f, BatchEntry &en) {
                       base_entry(f, en);
                       en.x = xsel(f);
                       return ctas_of(f);
                   });
    };
    auto per_256 = [](const BatchFit &f) { return (int)qmlg::ceil_div(f.n, 256); };
    auto one = [](const BatchFit &) { return 1; };
    int st = QMLG_OK;

    // ---- kernel matrices
    std::vector<qmlg::GaussItem> gi;
    for (BatchFit &f : fits) {
        const QmlgBatchProblem &q = *f.q;
        if (q.kind == QMLG_KIND_GAUSSIAN)
            gi.push_back(qmlg::GaussItem{q.X, q.ldx, f.n, q.sigma, q.K, (int64_t)f.n, f.row_k,
                                         q.status + 1});
    }
    st = qmlg::gauss_group_kernel_matrix(gi.data(), (int)gi.size(), d, b.kdig, b.kexp, b.knorm,
                                         b.maxbuf, RK, b.err, s);
    for (BatchFit &f : fits) {
        if (st != QMLG_OK) return st;
        const QmlgBatchProblem &q = *f.q;
        if (q.kind == QMLG_KIND_LAPLACIAN)
            st = qmlg_laplacian_kernel_fixed_async(q.X, q.ldx, f.n, q.X, q.ldx, f.n, d, q.sigma, q.K,
                                                   f.n, QMLG_KERNEL_SYMMETRIC, 0.0, q.status + 1,
                                                   f.lws, f.lws_bytes, stream);
    }
    if (st != QMLG_OK) return st;
    st = vec(kCopyDiag, per_256, [](const BatchFit &f) { return f.r; });
    if (st != QMLG_OK) return st;

    // ---- factorisation, lockstep over 64-column steps
    int maxn = 0;
    for (const BatchFit &f : fits) maxn = std::max(maxn, f.n);
    std::vector<qmlg::GroupItem> items;
    std::vector<qmlg::SliceItem> slices;
    for (int k0 = 0; k0 < maxn && st == QMLG_OK; k0 += NB) {
        const int kb = k0 / NB, r1 = k0 + NB, K0 = k0 / qmlg::NBO * qmlg::NBO;
        st = run([&](int grid) { potrf_group_kernel<<<grid, POTRF_THREADS, 0, s>>>(L.g); },
                 [&](const BatchFit &f, BatchEntry &en) {
                     if (f.n <= k0) return 0;
                     base_entry(f, en);
                     en.k = kb;
                     return 1;
                 });
        if (st != QMLG_OK) break;
        st = run([&](int grid) {
                     trsm_group_kernel<<<grid, 4 * trsm_rows, trsm_smem(trsm_rows), s>>>(
                         L.g, qmlg::kEmuMaxSlices, RT);
                 },
                 [&](const BatchFit &f, BatchEntry &en) {
                     if (f.n <= r1) return 0;
                     const int K1 = std::min(K0 + qmlg::NBO, f.n);
                     const bool inner = r1 < K1;
                     base_entry(f, en);
                     en.k = kb;
                     en.drows = inner ? std::min(qmlg::plane_rows(f.n),
                                                 (int)qmlg::ceil_div(f.n - r1, 128) * 128)
                                      : 0;
                     en.digits = inner ? b.idig + (size_t)f.row_p * NB : nullptr;
                     en.expo = inner ? b.iexp + f.row_p : nullptr;
                     const int rows = inner ? en.drows : f.n - r1;
                     return (int)qmlg::ceil_div(rows, trsm_rows);
                 });
        if (st != QMLG_OK) break;
        items.clear();
        for (const BatchFit &f : fits) {
            const int K1 = std::min(K0 + qmlg::NBO, f.n);
            if (f.n > r1 && r1 < K1)
                items.push_back(qmlg::GroupItem{f.q->K, (int64_t)f.n, r1, K1, r1, f.n, f.row_p,
                                                f.row_p, 0.0});
        }
        st = qmlg::emu_tc_group_update(items.data(), (int)items.size(), b.idig, b.iexp, NB, RT,
                                       qmlg::kEmuMaxSlices, b.err, s, tile_cols);
        if (st != QMLG_OK || r1 % qmlg::NBO != 0) continue;
        // the end of a 512-column panel: its digit planes, then every trailing update
        slices.clear();
        items.clear();
        for (const BatchFit &f : fits) {
            if (f.n <= r1) continue;
            slices.push_back(qmlg::SliceItem{f.q->K, (int64_t)f.n, r1, f.n - r1, K0, qmlg::NBO, f.row_p,
                                             f.q->status});
            items.push_back(qmlg::GroupItem{f.q->K, (int64_t)f.n, r1, f.n, r1, f.n, f.row_p,
                                            f.row_p, 0.0});
        }
        st = qmlg::slice_rows_group(slices.data(), (int)slices.size(), qmlg::NBO, RT,
                                    qmlg::kEmuMaxSlices, b.pdig, b.pexp, s);
        if (st == QMLG_OK)
            st = qmlg::emu_tc_group_update(items.data(), (int)items.size(), b.pdig, b.pexp, qmlg::NBO,
                                           RT, qmlg::kEmuMaxSlices, b.err, s, tile_cols);
    }
    if (st != QMLG_OK) return st;
    st = run([&](int grid) { invert_group_kernel<<<grid, 64, 0, s>>>(L.g); },
             [&](const BatchFit &f, BatchEntry &en) {
                 base_entry(f, en);
                 return f.nblk;
             });
    if (st != QMLG_OK) return st;

    // ---- solves: alpha = y, L L^T alpha = y, then refine_steps refinement steps
    int maxblk = 0;
    for (const BatchFit &f : fits) maxblk = std::max(maxblk, f.nblk);
    const int cap = 4 * std::max(1, qmlg::tc_sm_count());
    auto solve = [&](double *(*xsel)(const BatchFit &)) -> int {
        int rc = QMLG_OK;
        // one launch per pair of 64-row blocks and direction (en.k: the pair)
        const int maxsteps = (maxblk + 1) / 2;
        for (int t = 0; t < maxsteps && rc == QMLG_OK; ++t)
            rc = run([&](int grid) { fwd_group_kernel<<<grid, STEP_THREADS, 0, s>>>(L.g); },
                     [&](const BatchFit &f, BatchEntry &en) {
                         if (2 * t >= f.nblk) return 0;
                         base_entry(f, en);
                         en.x = xsel(f);
                         en.k = t;
                         return 1 + trsv_fwd_extra(f.n, t, cap);
                     });
        for (int u = 0; u < maxsteps && rc == QMLG_OK; ++u)
            rc = run([&](int grid) { bwd_group_kernel<<<grid, STEP_THREADS, 0, s>>>(L.g); },
                     [&](const BatchFit &f, BatchEntry &en) {
                         if (2 * u >= f.nblk) return 0;
                         base_entry(f, en);
                         en.x = xsel(f);
                         en.k = u;
                         return 1 + trsv_bwd_extra(f.n, u, cap);
                     });
        return rc;
    };
    auto sel_alpha = [](const BatchFit &f) { return f.q->alpha; };
    auto sel_r = [](const BatchFit &f) { return f.r; };
    st = vec(kCopyY, per_256, sel_alpha);
    if (st == QMLG_OK) st = solve(sel_alpha);
    for (int it = 0; it < refine_steps && st == QMLG_OK; ++it) {
        st = run([&](int grid) { symv_group_kernel<<<grid, 256, RES_SMEM, s>>>(L.g); },
                 [&](const BatchFit &f, BatchEntry &en) {
                     base_entry(f, en);
                     en.x = f.q->alpha;
                     return (int)(qmlg::ceil_div(f.n, RES_ROWS) * qmlg::ceil_div(f.n, RES_CHUNK));
                 });
        if (st == QMLG_OK)
            st = run([&](int grid) { finish_group_kernel<<<grid, 256, 0, s>>>(L.g); },
                     [&](const BatchFit &f, BatchEntry &en) {
                         base_entry(f, en);
                         en.x = f.q->alpha;
                         return (int)qmlg::ceil_div(f.n, 256);
                     });
        if (st == QMLG_OK) st = solve(sel_r);
        if (st == QMLG_OK) st = vec(kZeroSums, one, sel_alpha);
        if (st == QMLG_OK)
            st = run([&](int grid) { axpy_group_kernel<<<grid, 256, 0, s>>>(L.g); },
                     [&](const BatchFit &f, BatchEntry &en) {
                         base_entry(f, en);
                         en.x = f.q->alpha;
                         return (int)qmlg::ceil_div(f.n, 256);
                     });
    }
    if (st == QMLG_OK) st = vec(kFinishFlags, one, sel_alpha);
    return st;
}
