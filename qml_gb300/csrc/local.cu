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
#include <vector>

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

// ---- local kernels from atom-pair kernel matrices (tensor cores / fixed point) --
//
// For each sigma and each chunk of A's molecules, the atom-pair matrix
// Ka[j, i] = k(A_j, B_i) of the chunk's atoms against all of B's comes from the
// Gaussian tensor-core kernel (qmlg_gaussian_kernel_emulated) or the fixed-point
// Laplacian (qmlg_laplacian_kernel_fixed), column-major in the workspace.  Two
// reductions then give the molecule pairs: R[j, b] = sum over B-molecule b's atoms
// (one thread per row j, so a warp reads 32 consecutive doubles of a column), and
// K[s, a, b] = sum over A-molecule a's rows of R.  Every term is positive, so each
// K entry keeps the per-entry relative bound of the atom-pair kernel.

namespace {

constexpr int64_t kLocalPairBytes = 2ll << 30;  // atom-pair matrix per chunk
constexpr int64_t kLocalMinRows = 4096;         // rows a chunk may always hold

int64_t local_chunk_rows(int64_t natoms_a, int64_t natoms_b)
{
    int64_t r = kLocalPairBytes / (8 * (natoms_b < 1 ? 1 : natoms_b));
    if (r < kLocalMinRows) r = kLocalMinRows;
    if (r > 65535ll * 256) r = 65535ll * 256;  // the row-sum grid's y extent
    return r < natoms_a ? r : (natoms_a < 1 ? 1 : natoms_a);
}

// B molecules mb0, mb0 + 1, ...; the atom-pair matrix starts at B atom col0.
__global__ void local_rowsum_kernel(const double *__restrict__ Ka, int64_t ldka, int rows,
                                    const int64_t *__restrict__ offb, int mb0, int64_t col0,
                                    double *__restrict__ R, int64_t ldr)
{
    const int mb = mb0 + blockIdx.x;
    const int j = blockIdx.y * blockDim.x + threadIdx.x;
    if (j >= rows) return;
    const int64_t i0 = offb[mb] - col0, i1 = offb[mb + 1] - col0;
    double acc = 0.0;
    for (int64_t i = i0; i < i1; ++i) acc += Ka[j + ldka * i];
    R[j + ldr * (mb - mb0)] = acc;
}

// A molecules ma0 .. ma0 + cnt - 1 against B molecules mb0 .. nm2 - 1.
__global__ void local_segsum_kernel(const double *__restrict__ R, int64_t ldr,
                                    const int64_t *__restrict__ offa, int ma0, int cnt, int nm1,
                                    int mb0, int nm2, int ns, int si, double *__restrict__ K)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (int64_t)cnt * (nm2 - mb0)) return;
    const int ma = ma0 + (int)(t % cnt);
    const int mb = mb0 + (int)(t / cnt);
    const int64_t base = offa[ma0];
    const int64_t j0 = offa[ma] - base, j1 = offa[ma + 1] - base;
    double acc = 0.0;
    for (int64_t j = j0; j < j1; ++j) acc += R[j + ldr * (mb - mb0)];
    K[si + (int64_t)ns * (ma + (int64_t)nm1 * mb)] = acc;
}

// Symmetric mode: K[s, b, a] = K[s, a, b] for b > a.  The two sums run over the
// same terms in a different order, so the copy makes K exactly symmetric.
__global__ void local_mirror_kernel(double *__restrict__ K, int nm, int ns)
{
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t per = (int64_t)nm * nm;
    if (t >= per * ns) return;
    const int si = (int)(t % ns);
    const int64_t ab = t / ns;
    const int a = (int)(ab % nm), b = (int)(ab / nm);
    if (b > a) K[si + (int64_t)ns * (b + (int64_t)nm * a)] = K[si + (int64_t)ns * (a + (int64_t)nm * b)];
}

size_t local_inner_ws(int kind, int64_t rows, int64_t natoms_b, int d)
{
    return kind == 0 ? qmlg_gaussian_kernel_emulated_workspace_size((int)rows, (int)natoms_b, d, 0)
                     : qmlg_laplacian_kernel_fixed_workspace_size((int)rows, (int)natoms_b, d, 0);
}

}  // namespace

extern "C" size_t qmlg_local_kernels_emulated_workspace_size(int kind, int64_t natoms_a,
                                                             int64_t natoms_b, int nm2, int d)
{
    const int64_t rows = local_chunk_rows(natoms_a, natoms_b);
    qmlg::WorkspacePlan p;
    p.add<double>((size_t)rows * (size_t)(natoms_b < 1 ? 1 : natoms_b));
    p.add<double>((size_t)rows * (size_t)(nm2 < 1 ? 1 : nm2));
    p.add<char>(local_inner_ws(kind, rows, natoms_b, d));
    return p.total();
}

extern "C" int qmlg_local_kernels_emulated(int kind, const double *A, int64_t lda,
                                           const int64_t *offsets_a, int nm1, const double *B,
                                           int64_t ldb, const int64_t *offsets_b, int nm2, int d,
                                           const double *sigmas, int nsigmas, double *K, int flags,
                                           void *workspace, size_t ws_bytes, void *stream)
{
    if ((kind != 0 && kind != 1) || nm1 < 0 || nm2 < 0 || d < 0 || nsigmas < 0) return QMLG_E_ARG;
    if (nm1 == 0 || nm2 == 0 || nsigmas == 0) return QMLG_OK;
    if (A == nullptr || B == nullptr || offsets_a == nullptr || offsets_b == nullptr ||
        sigmas == nullptr || K == nullptr || lda < d || ldb < d)
        return QMLG_E_ARG;
    const bool symmetric = (flags & QMLG_KERNEL_SYMMETRIC) != 0;
    if (symmetric && (nm1 != nm2 || A != B || lda != ldb || offsets_a != offsets_b)) return QMLG_E_ARG;
    cudaStream_t s = qmlg::as_stream(stream);
    // the offsets and sigmas steer the host loop
    std::vector<int64_t> oa(nm1 + 1), ob(nm2 + 1);
    std::vector<double> sg(nsigmas);
    cudaError_t e = cudaMemcpyAsync(oa.data(), offsets_a, sizeof(int64_t) * (nm1 + 1),
                                    cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(ob.data(), offsets_b, sizeof(int64_t) * (nm2 + 1), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sg.data(), sigmas, sizeof(double) * nsigmas, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return qmlg::set_cuda_error(e);
    if (oa[0] != 0 || ob[0] != 0) return QMLG_E_ARG;
    for (int m = 0; m < nm1; ++m)
        if (oa[m + 1] < oa[m]) return QMLG_E_ARG;
    for (int m = 0; m < nm2; ++m)
        if (ob[m + 1] < ob[m]) return QMLG_E_ARG;
    const int64_t nat_a = oa[nm1], nat_b = ob[nm2];
    if (nat_a > 0x7fffffffll || nat_b > 0x7fffffffll) return QMLG_E_TOO_LARGE;
    if (ws_bytes < qmlg_local_kernels_emulated_workspace_size(kind, nat_a, nat_b, nm2, d))
        return QMLG_E_WORKSPACE;
    const int64_t rows_max = local_chunk_rows(nat_a, nat_b);
    if (nat_a == 0 || nat_b == 0) {
        // molecules without atoms: every sum is empty
        e = cudaMemsetAsync(K, 0, sizeof(double) * (size_t)nsigmas * nm1 * nm2, s);
        return e == cudaSuccess ? QMLG_OK : qmlg::set_cuda_error(e);
    }
    qmlg::Workspace ws(workspace, ws_bytes);
    double *Ka = ws.take<double>((size_t)rows_max * (size_t)nat_b);
    double *R = ws.take<double>((size_t)rows_max * (size_t)nm2);
    const size_t inner_bytes = local_inner_ws(kind, rows_max, nat_b, d);
    char *inner = ws.take<char>(inner_bytes);
    if (!Ka || !R || !inner) return QMLG_E_WORKSPACE;
    // one chunk covering every atom of a symmetric problem takes the symmetric kernel;
    // with several, a chunk of a symmetric problem starts at its own first atom and
    // molecule on the B side (the pairs before them come from the mirror)
    const bool sym_chunk = symmetric && rows_max >= nat_a;
    for (int si = 0; si < nsigmas; ++si) {
        if (!(sg[si] > 0.0) || !std::isfinite(sg[si])) return QMLG_E_ARG;
        int ma0 = 0;
        while (ma0 < nm1) {
            int ma1 = ma0;
            while (ma1 < nm1 && oa[ma1 + 1] - oa[ma0] <= rows_max) ++ma1;
            if (ma1 == ma0) return QMLG_E_TOO_LARGE;  // one molecule above the chunk rows
            const int64_t r0 = oa[ma0];
            const int rows = (int)(oa[ma1] - r0);
            const int mb0 = symmetric ? ma0 : 0;      // first B molecule of this chunk
            const int64_t c0 = symmetric ? r0 : 0;    // its first atom
            const int cols = (int)(nat_b - c0);
            int st = QMLG_OK;
            if (rows > 0) {
                const double *Ac = A + r0 * lda;
                const double *Bc = symmetric ? Ac : B;
                const int fl = sym_chunk ? QMLG_KERNEL_SYMMETRIC : 0;
                st = kind == 0
                         ? qmlg_gaussian_kernel_emulated(Ac, lda, rows, Bc, symmetric ? lda : ldb, cols,
                                                         d, sg[si], Ka, rows, fl, 0.0, inner,
                                                         inner_bytes, stream)
                         : qmlg_laplacian_kernel_fixed(Ac, lda, rows, Bc, symmetric ? lda : ldb, cols,
                                                       d, sg[si], Ka, rows, fl, 0.0, inner, inner_bytes,
                                                       stream);
                if (st != QMLG_OK) return st;
                local_rowsum_kernel<<<dim3((unsigned)(nm2 - mb0), (unsigned)qmlg::ceil_div(rows, 256)),
                                      256, 0, s>>>(Ka, rows, rows, offsets_b, mb0, c0, R, rows);
                qmlg::count_launches(1);
                st = qmlg::check_launch();
                if (st != QMLG_OK) return st;
            }
            const int cnt = ma1 - ma0;
            const int64_t pairs = (int64_t)cnt * (nm2 - mb0);
            local_segsum_kernel<<<(unsigned)qmlg::ceil_div(pairs, 256), 256, 0, s>>>(
                R, rows > 0 ? rows : 1, offsets_a, ma0, cnt, nm1, mb0, nm2, nsigmas, si, K);
            qmlg::count_launches(1);
            st = qmlg::check_launch();
            if (st != QMLG_OK) return st;
            ma0 = ma1;
        }
    }
    if (symmetric && nm1 > 1) {
        const int64_t total = (int64_t)nm1 * nm1 * nsigmas;
        local_mirror_kernel<<<(unsigned)qmlg::ceil_div(total, 256), 256, 0, s>>>(K, nm1, nsigmas);
        qmlg::count_launches(1);
        return qmlg::check_launch();
    }
    return QMLG_OK;
}
