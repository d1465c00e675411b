// Emulated-FP64 trailing update of the blocked Cholesky on the bf16 tensor cores.
//
// The panel P (rows k1..n of the nb = 64 columns just factorised) is cut into S
// base-128 digit planes per row (see emulated_gemm.cuh), then every 64 x 64 tile
// of the trailing lower triangle computes
//     C[i][j] -= 2^(e_i + e_j) * sum_l 128^-(l+2) * sum_{s+t=l} D_s[i,:] . D_t[j,:]
// with mma.sync m16n8k16 bf16 -> FP32 (exact: |partial| <= 8 * 64 * 4096 < 2^24),
// the levels merged in two 64-bit integers and converted to FP64 once.
#include <cmath>

#include "emulated_gemm.cuh"

namespace {

constexpr int TILE = 64;
constexpr int KP = 64;        // panel width (digits per row per plane)
constexpr int KS = KP + 8;    // padded smem row, conflict-free fragment loads

// One warp per panel row: exponent and digit planes.
__global__ void slice_panel_kernel(const double *__restrict__ A, int64_t lda, int n, int k0,
                                   int nb, int k1, int slices, __nv_bfloat16 *__restrict__ digits,
                                   int *__restrict__ expo, const int *__restrict__ info)
{
    if (*info != 0) return;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const int row = k1 + warp;
    if (row >= n) return;
    double v0 = 0.0, v1 = 0.0;
    if (lane < nb) v0 = A[(int64_t)row * lda + k0 + lane];
    if (lane + 32 < nb) v1 = A[(int64_t)row * lda + k0 + lane + 32];
    double m = fmax(fabs(v0), fabs(v1));
    for (int off = 16; off > 0; off >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, off));
    int e = 0;
    if (m > 0.0 && isfinite(m)) {
        frexp(m, &e);
        e += 1;  // |x| * 2^-e < 1/2
    }
    v0 = ldexp(v0, -e);
    v1 = ldexp(v1, -e);
    const int64_t plane = (int64_t)n * KP;
    __nv_bfloat16 *dst = digits + (int64_t)row * KP;
    for (int s = 0; s < slices; ++s) {
        v0 *= 128.0;
        v1 *= 128.0;
        const double d0 = rint(v0), d1 = rint(v1);
        v0 -= d0;
        v1 -= d1;
        dst[(int64_t)s * plane + lane] = __double2bfloat16(d0);
        dst[(int64_t)s * plane + lane + 32] = __double2bfloat16(d1);
    }
    if (lane == 0) expo[row] = e;
}

__device__ __forceinline__ void tri_index(int64_t t, int &bi, int &bj)
{
    int64_t r = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > t) --r;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    bi = (int)r;
    bj = (int)(t - r * (r + 1) / 2);
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ double pow2(int e)
{
    // 2^e for normal exponents
    return __longlong_as_double((long long)(e + 1023) << 52);
}

// 64 x 64 tile, 8 warps as 2 (rows) x 4 (cols), 32 x 16 outputs per warp.
__global__ void __launch_bounds__(256)
emu_syrk_kernel(double *__restrict__ A, int64_t lda, int n, int k1, int slices,
                const __nv_bfloat16 *__restrict__ digits, const int *__restrict__ expo,
                const int *__restrict__ info)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if (*info != 0) return;
    __nv_bfloat16 *As = reinterpret_cast<__nv_bfloat16 *>(smem_raw);
    __nv_bfloat16 *Bs = As + (size_t)slices * TILE * KS;
    int bi, bj;
    tri_index(blockIdx.x, bi, bj);
    const int i0 = k1 + bi * TILE, j0 = k1 + bj * TILE;
    const int tid = threadIdx.x;
    const int64_t plane = (int64_t)n * KP;

    // digit planes of the tile's rows (i) and columns (j): 16-byte vectors
    for (int e = tid; e < slices * TILE * (KP / 8); e += 256) {
        const int s = e / (TILE * (KP / 8));
        const int rem = e % (TILE * (KP / 8));
        const int r = rem / (KP / 8), v = rem % (KP / 8);
        uint4 za = make_uint4(0, 0, 0, 0), zb = make_uint4(0, 0, 0, 0);
        if (i0 + r < n)
            za = *reinterpret_cast<const uint4 *>(digits + s * plane + (int64_t)(i0 + r) * KP + v * 8);
        if (j0 + r < n)
            zb = *reinterpret_cast<const uint4 *>(digits + s * plane + (int64_t)(j0 + r) * KP + v * 8);
        *reinterpret_cast<uint4 *>(As + ((size_t)s * TILE + r) * KS + v * 8) = za;
        *reinterpret_cast<uint4 *>(Bs + ((size_t)s * TILE + r) * KS + v * 8) = zb;
    }
    __syncthreads();

    const int warp = tid >> 5, lane = tid & 31;
    const int wm = warp >> 2, wn = warp & 3;
    const int g = lane >> 2, c = lane & 3;
    const int H = (slices + 1) / 2;
    long long hi[2][2][4], lo[2][2][4];
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int q = 0; q < 4; ++q) hi[a][b][q] = lo[a][b][q] = 0;

    for (int l = 0; l < slices; ++l) {
        float acc[2][2][4];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[a][b][q] = 0.f;
        for (int s = 0; s <= l; ++s) {
            const int t = l - s;
            const __nv_bfloat16 *Ap = As + (size_t)s * TILE * KS;
            const __nv_bfloat16 *Bp = Bs + (size_t)t * TILE * KS;
#pragma unroll
            for (int k0 = 0; k0 < KP; k0 += 16) {
                uint32_t af[2][4];
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const int r = wm * 32 + a * 16 + g;
                    af[a][0] = *reinterpret_cast<const uint32_t *>(Ap + r * KS + k0 + 2 * c);
                    af[a][1] = *reinterpret_cast<const uint32_t *>(Ap + (r + 8) * KS + k0 + 2 * c);
                    af[a][2] = *reinterpret_cast<const uint32_t *>(Ap + r * KS + k0 + 2 * c + 8);
                    af[a][3] = *reinterpret_cast<const uint32_t *>(Ap + (r + 8) * KS + k0 + 2 * c + 8);
                }
#pragma unroll
                for (int b = 0; b < 2; ++b) {
                    const int col = wn * 16 + b * 8 + g;
                    const uint32_t b0 = *reinterpret_cast<const uint32_t *>(Bp + col * KS + k0 + 2 * c);
                    const uint32_t b1 = *reinterpret_cast<const uint32_t *>(Bp + col * KS + k0 + 2 * c + 8);
#pragma unroll
                    for (int a = 0; a < 2; ++a) mma_bf16(acc[a][b], af[a], b0, b1);
                }
            }
        }
        // merge the level: exact integers, base 128
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 2; ++b)
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const long long v = (long long)__float2int_rn(acc[a][b][q]);
                    if (l < H) hi[a][b][q] = hi[a][b][q] * 128 + v;
                    else lo[a][b][q] = lo[a][b][q] * 128 + v;
                }
    }

    const double shi = pow2(-7 * (H + 1)), slo = pow2(-7 * (slices + 1));
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int i = i0 + wm * 32 + a * 16 + g + ((q & 2) ? 8 : 0);
                const int j = j0 + wn * 16 + b * 8 + 2 * c + (q & 1);
                if (i < n && j < n && j <= i) {
                    const double t = fma((double)hi[a][b][q], shi, (double)lo[a][b][q] * slo);
                    const double v = ldexp(t, expo[i] + expo[j]);
                    A[(int64_t)i * lda + j] -= v;
                }
            }
}

}  // namespace

namespace qmlg {

int emu_trailing_update(double *A, int64_t lda, int n, int k0, int nb, int slices,
                        __nv_bfloat16 *digits, int *expo, const int *d_info, cudaStream_t s)
{
    if (slices < 1 || slices > kEmuMaxSlices || nb > KP) return QMLG_E_ARG;
    const int k1 = k0 + nb;
    const int rows = n - k1;
    if (rows <= 0) return QMLG_OK;
    { slice_panel_kernel<<<(int)ceil_div((int64_t)rows * 32, 256), 256, 0, s>>>(
        A, lda, n, k0, nb, k1, slices, digits, expo, d_info); qmlg::count_launches(1); }
    const int64_t t = ceil_div(rows, TILE);
    const size_t smem = (size_t)2 * slices * TILE * KS * sizeof(__nv_bfloat16);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(emu_syrk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)((size_t)2 * kEmuMaxSlices * TILE * KS * sizeof(__nv_bfloat16)));
        attr_set = true;
    }
    { emu_syrk_kernel<<<(unsigned)(t * (t + 1) / 2), 256, smem, s>>>(A, lda, n, k1, slices, digits,
                                                                   expo, d_info); qmlg::count_launches(1); }
    return check_launch();
}

}  // namespace qmlg
