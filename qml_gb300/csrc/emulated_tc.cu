// Emulated-FP64 products on the tcgen05 tensor cores (sm_103a).
//
//   C[i][j]  -=  sum_k P[i][k] * Q[j][k]        (mode SUBTRACT, C row-major, FP64)
//
// for an (i, j) region, where the rows of P and Q were cut into S base-128 digit
// planes by slice_rows_kernel (|digit| <= 64, exact in bf16) with one power-of-two
// scale per row.  Level l = s + t of the digit products is accumulated exactly in
// FP32 in tensor memory:
//   TMEM lane   = j (128 per tile; the contiguous index of C, so stores coalesce)
//   TMEM column = l * 64 + (i - i0)   (64 per level, 8 levels = all 512 columns)
// A tile runs kchunks 64-deep K chunks.  Per chunk the 8 digit planes of the 64 i-rows
// are loaded once (double-buffered) and the 8 planes of the 128 j-rows stream
// through a 3-slot ring; each j-plane s meets the i-planes t <= S-1-s.
// Exactness: a level sums at most 8 * (64*kchunks) * 4096 products, so kchunks <= 8
// keeps every partial sum below 2^24.
//
// Warp roles (192 threads): warp 0 issues TMA loads, warp 1 owns TMEM and issues
// the MMAs from one thread, warps 2-5 (one per TMEM lane quarter) run the epilogue:
// the levels are merged in 64-bit integers, converted once to FP64, scaled by
// 2^(e_i + e_j) and subtracted from C.  Waits are bounded; a timeout sets *err.
#include <cuda.h>

#include <cmath>
#include <mutex>

#include "common.cuh"
#include "emulated_gemm.cuh"
#include "tc_ptx.cuh"

namespace {

using namespace qmlg::tc;

constexpr int TM = 128;         // TMEM lanes per tile (j)
constexpr int TN = 64;          // columns per level (i)
constexpr int KC = 64;          // K chunk: one 128-byte swizzled row of bf16
constexpr int S_MAX = 8;
constexpr int A_STAGES = 3;
constexpr int A_BYTES = TM * KC * 2;  // 16 KB
constexpr int B_BYTES = TN * KC * 2;  // 8 KB
constexpr int SMEM_BYTES = 2 * S_MAX * B_BYTES + A_STAGES * A_BYTES + 1024 /*align*/ + 256;

struct TileArgs {
    double *C;
    int64_t ldc;
    int jbase, jend;   // lanes: C column index range
    int ibase, iend;   // TMEM columns: C row index range
    int a_row0;        // digit row of j = jbase
    int b_row0;        // digit row of i = ibase
    int kchunks;
    int slices;
    const int *expA;   // per digit row
    const int *expB;
    int lower;         // update only j <= i
    int *err;
};

__device__ __forceinline__ double pow2i(int e)
{
    if (e >= -1022 && e <= 1023) return __longlong_as_double((long long)(e + 1023) << 52);
    return ldexp(1.0, e);
}

__global__ void __launch_bounds__(192, 1)
emu_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
              TileArgs p)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char *base =
        (unsigned char *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char *Bbuf = base;                               // [2][S_MAX][B_BYTES]
    unsigned char *Aring = base + 2 * S_MAX * B_BYTES;        // [A_STAGES][A_BYTES]
    uint64_t *bars = (uint64_t *)(Aring + A_STAGES * A_BYTES);
    uint64_t *bFull = bars, *bEmpty = bars + 2, *aFull = bars + 4, *aEmpty = bars + 7,
             *done = bars + 10;
    uint32_t *tmem_holder = (uint32_t *)(bars + 12);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j0 = p.jbase + blockIdx.x * TM;
    const int i0 = p.ibase + blockIdx.y * TN;
    const int ilast = min(i0 + TN, p.iend) - 1;
    if (p.lower && j0 > ilast) return;  // tile entirely above the diagonal
    const int S = p.slices;
    const int arow = p.a_row0 + (j0 - p.jbase);
    const int brow = p.b_row0 + (i0 - p.ibase);

    if (threadIdx.x == 0) {
        mbar_init(&bFull[0], 1);
        mbar_init(&bFull[1], 1);
        mbar_init(&bEmpty[0], 1);
        mbar_init(&bEmpty[1], 1);
        for (int k = 0; k < A_STAGES; ++k) {
            mbar_init(&aFull[k], 1);
            mbar_init(&aEmpty[k], 1);
        }
        mbar_init(done, 1);
        fence_barrier_init();
    }
    if (warp == 0 && lane == 0) {
        prefetch_tensormap(&mapA);
        prefetch_tensormap(&mapB);
    }
    if (warp == 1) tmem_alloc(tmem_holder, 512);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tmem_holder;

    if (warp == 0) {
        if (lane == 0) {
            // ---------------- TMA producer
            int it = 0;
            bool ok = true;
            for (int c = 0; c < p.kchunks && ok; ++c) {
                const int bb = c & 1;
                if (c >= 2 && !mbar_wait(&bEmpty[bb], ((c >> 1) - 1) & 1)) {
                    ok = false;
                    break;
                }
                mbar_expect_tx(&bFull[bb], (uint32_t)(S * B_BYTES));
                for (int t = 0; t < S; ++t)
                    tma_load_3d(Bbuf + (bb * S_MAX + t) * B_BYTES, &mapB, &bFull[bb], c * KC, brow, t);
                for (int s = 0; s < S; ++s, ++it) {
                    const int st = it % A_STAGES, round = it / A_STAGES;
                    if (round >= 1 && !mbar_wait(&aEmpty[st], (round - 1) & 1)) {
                        ok = false;
                        break;
                    }
                    mbar_expect_tx(&aFull[st], (uint32_t)A_BYTES);
                    tma_load_3d(Aring + st * A_BYTES, &mapA, &aFull[st], c * KC, arow, s);
                }
            }
            if (!ok) atomicOr(p.err, 1);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---------------- MMA issuer
            const uint32_t idesc = idesc_bf16_f32(TM, TN);
            int it = 0;
            bool ok = true;
            for (int c = 0; c < p.kchunks && ok; ++c) {
                const int bb = c & 1;
                if (!mbar_wait(&bFull[bb], (c >> 1) & 1)) {
                    ok = false;
                    break;
                }
                fence_after_sync();
                for (int s = 0; s < S; ++s, ++it) {
                    const int st = it % A_STAGES, round = it / A_STAGES;
                    if (!mbar_wait(&aFull[st], round & 1)) {
                        ok = false;
                        break;
                    }
                    fence_after_sync();
                    const uint64_t da = desc_sw128(Aring + st * A_BYTES);
                    for (int t = 0; t + s < S; ++t) {
                        const uint64_t db = desc_sw128(Bbuf + (bb * S_MAX + t) * B_BYTES);
                        const uint32_t dst = tmem + (uint32_t)((s + t) * TN);
#pragma unroll
                        for (int kk = 0; kk < KC / 16; ++kk) {
                            const uint32_t acc = (c > 0 || s > 0 || kk > 0) ? 1u : 0u;
                            mma_bf16(dst, da + (uint64_t)(kk * 2), db + (uint64_t)(kk * 2), idesc, acc);
                        }
                    }
                    mma_commit(&aEmpty[st]);
                }
                mma_commit(&bEmpty[bb]);
            }
            if (!ok) atomicOr(p.err, 2);
            mma_commit(done);
        }
    } else {
        // ---------------- epilogue: warps 2..5 -> TMEM lane quarters 2,3,0,1
        const int q = warp & 3;
        const int jl = q * 32 + lane;
        const int j = j0 + jl;
        bool ok = mbar_wait(done, 0);
        if (!ok && lane == 0) atomicOr(p.err, 4);
        fence_after_sync();
        const int ej = (j < p.jend) ? p.expA[arow + jl] : 0;
        const int H = (S + 1) / 2;
        const int lo_levels = S - H;
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
        for (int g = 0; g < TN / 16; ++g) {
            uint32_t v[S_MAX][16];
#pragma unroll
            for (int l = 0; l < S_MAX; ++l)
                if (l < S) tmem_ld16(lane_base + (uint32_t)(l * TN + g * 16), v[l]);
            tmem_ld_wait();
            if (!ok) continue;
#pragma unroll
            for (int col = 0; col < 16; ++col) {
                const int il = g * 16 + col;
                const int i = i0 + il;
                long long hi = 0, lo = 0;
#pragma unroll
                for (int l = 0; l < S_MAX; ++l) {
                    if (l >= S) break;
                    const long long d = (long long)__float2int_rn(__uint_as_float(v[l][col]));
                    if (l < H) hi = hi * 128 + d;
                    else lo = lo * 128 + d;
                }
                // value = hi * 128^lo_levels + lo, kept in 62 bits by dropping the lowest
                // `shift` bits of lo (far below FP64 resolution of the value)
                const int shift = lo_levels >= 2 ? 12 : 0;
                const long long v64 = (hi << (7 * lo_levels - shift)) + (lo >> shift);
                if (j < p.jend && i < p.iend && (!p.lower || j <= i)) {
                    const int ei = p.expB[brow + il];
                    const double scale = pow2i(ei + ej + shift - 7 * (S + 1));
                    double *cp = p.C + (int64_t)i * p.ldc + j;
                    *cp = fma(-(double)v64, scale, *cp);
                }
            }
        }
    }
    fence_before_sync();
    __syncthreads();
    if (warp == 1) tmem_dealloc(tmem, 512);
}

// One warp per row: power-of-two row scale over the K-range and S digit planes.
// src rows r0 .. r0+nrows-1, columns c0 .. c0+kw-1 of the row-major matrix;
// digits [S][rpad][kp] bf16 (zero beyond kw and beyond nrows), expo [rpad].
__global__ void slice_rows_kernel(const double *__restrict__ A, int64_t lda, int r0, int nrows,
                                  int c0, int kw, int kp, int rpad, int slices,
                                  __nv_bfloat16 *__restrict__ digits, int *__restrict__ expo,
                                  const int *__restrict__ info)
{
    if (info != nullptr && *info != 0) return;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= rpad) return;
    const bool live = warp < nrows;
    const double *row = A + (int64_t)(r0 + warp) * lda + c0;
    double m = 0.0;
    if (live)
        for (int k = lane; k < kw; k += 32) m = fmax(m, fabs(row[k]));
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    int e = 0;
    if (m > 0.0 && isfinite(m)) {
        frexp(m, &e);
        e += 1;  // |x| * 2^-e < 1/2
    }
    const int64_t plane = (int64_t)rpad * kp;
    __nv_bfloat16 *dst = digits + (int64_t)warp * kp;
    for (int k = lane; k < kp; k += 32) {
        double v = (live && k < kw) ? ldexp(row[k], -e) : 0.0;
        for (int s = 0; s < slices; ++s) {
            v *= 128.0;
            const double d = rint(v);
            v -= d;
            dst[(int64_t)s * plane + k] = __double2bfloat16(d);
        }
    }
    if (lane == 0) expo[warp] = e;
}

typedef CUresult (*EncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                             const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                             const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                             CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeFn encode_fn()
{
    static EncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeFn>(p);
    });
    return fn;
}

int make_plane_map(CUtensorMap *map, const __nv_bfloat16 *digits, int kp, int rpad, int slices,
                   int box_rows)
{
    EncodeFn fn = encode_fn();
    if (fn == nullptr) return QMLG_E_CUDA;
    cuuint64_t dims[3] = {(cuuint64_t)kp, (cuuint64_t)rpad, (cuuint64_t)slices};
    cuuint64_t strides[2] = {(cuuint64_t)kp * 2, (cuuint64_t)rpad * kp * 2};
    cuuint32_t box[3] = {(cuuint32_t)KC, (cuuint32_t)box_rows, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, (void *)digits, dims, strides, box,
                    es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? QMLG_OK : QMLG_E_CUDA;
}

}  // namespace

namespace qmlg {

int slice_rows(const double *A, int64_t lda, int r0, int nrows, int c0, int kw, int kp, int rpad,
               int slices, __nv_bfloat16 *digits, int *expo, const int *d_info, cudaStream_t s)
{
    if (slices < 1 || slices > S_MAX || kp % KC != 0 || kw > kp || nrows > rpad) return QMLG_E_ARG;
    slice_rows_kernel<<<(unsigned)ceil_div((int64_t)rpad * 32, 256), 256, 0, s>>>(
        A, lda, r0, nrows, c0, kw, kp, rpad, slices, digits, expo, d_info);
    count_launches(1);
    return check_launch();
}

int emu_tc_update(double *C, int64_t ldc, int jbase, int jend, int ibase, int iend,
                  const __nv_bfloat16 *digits, const int *expo, int kp, int rpad, int slices,
                  int a_row0, int b_row0, int lower, int *d_err, cudaStream_t s)
{
    if (jend <= jbase || iend <= ibase) return QMLG_OK;
    if (slices < 1 || slices > S_MAX || kp % KC != 0 || kp / KC > 8) return QMLG_E_ARG;
    CUtensorMap mA, mB;
    int st = make_plane_map(&mA, digits, kp, rpad, slices, TM);
    if (st == QMLG_OK) st = make_plane_map(&mB, digits, kp, rpad, slices, TN);
    if (st != QMLG_OK) return st;
    static std::once_flag attr_once;
    std::call_once(attr_once, [] {
        cudaFuncSetAttribute(emu_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             SMEM_BYTES);
    });
    TileArgs a{C, ldc, jbase, jend, ibase, iend, a_row0, b_row0, kp / KC, slices,
               expo, expo, lower, d_err};
    dim3 grid((unsigned)ceil_div(jend - jbase, TM), (unsigned)ceil_div(iend - ibase, TN));
    emu_tc_kernel<<<grid, 192, SMEM_BYTES, s>>>(mA, mB, a);
    count_launches(1);
    return check_launch();
}

}  // namespace qmlg
