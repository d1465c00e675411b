// Sorted Coulomb matrix: one warp per molecule.
//
// Restates fgenerate_coulomb_matrix (qml/frepresentations.f90:52-140) with the
// reference's single-thread arithmetic so that every value and the permutation are
// bit-identical to it:
//   M_ii = 0.5 * Z_i^2.4, with Z^2.4 taken from a host pow() table for integer
//          charges 0..127 (device pow is not guaranteed to round like the host's);
//   M_ij = (Z_i * Z_j) / sqrt((dx*dx + dy*dy) + dz*dz), no FMA contraction;
//   row norm_i = M_ii^2, then + M_ij^2 over j ascending, j != i;
//   order: natoms rounds of "first index of the minimum row norm" (a warp argmin
//          by shuffles, ties to the lower lane), the winner placed at the end of
//          the order and its norm replaced by DBL_MAX, as at :116-121;
//   output: packed lower triangle cm[m(m+1)/2 + n] = M[s_m][s_n], zero-filled.
// Lane i owns atom i, so molecules have at most 32 atoms (QM7 has at most 23).
#include <cfloat>
#include <cmath>
#include <mutex>

#include "common.cuh"

namespace {

constexpr int kWarpsPerBlock = 4;
constexpr int kMaxAtoms = 32;
constexpr int kZTable = 128;

__constant__ double c_zpow[kZTable];

__global__ void __launch_bounds__(kWarpsPerBlock * 32)
coulomb_kernel(const double *__restrict__ charges, const double *__restrict__ coords,
               const int64_t *__restrict__ offsets, int n_mol, int size, int sorting,
               double *__restrict__ out, int *__restrict__ status)
{
    __shared__ double s_m[kWarpsPerBlock][kMaxAtoms][kMaxAtoms + 1];
    __shared__ int s_order[kWarpsPerBlock][kMaxAtoms];

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    const int mol = blockIdx.x * kWarpsPerBlock + warp;
    if (mol >= n_mol) return;

    const int64_t first = offsets[mol];
    const int natoms = (int)(offsets[mol + 1] - first);
    const int64_t len = (int64_t)size * (size + 1) / 2;
    double *dst = out + (int64_t)mol * len;

    if (natoms > size || natoms > kMaxAtoms || natoms < 0) {
        if (lane == 0 && status != nullptr) atomicMin(status, QMLG_E_TOO_MANY_ATOMS);
        for (int64_t e = lane; e < len; e += 32) dst[e] = 0.0;
        return;
    }

    const bool live = lane < natoms;
    double z = 0.0, x = 0.0, y = 0.0, w = 0.0;
    if (live) {
        z = charges[first + lane];
        x = coords[3 * (first + lane) + 0];
        y = coords[3 * (first + lane) + 1];
        w = coords[3 * (first + lane) + 2];
    }
    double zp;
    const int zi = (int)z;
    if ((double)zi == z && zi >= 0 && zi < kZTable) {
        zp = c_zpow[zi];
    } else {
        zp = pow(z, 2.4);
    }
    const double diag = __dmul_rn(0.5, zp);

    // Row i of M into shared memory, row norm in the reference's order.
    double norm = __dmul_rn(diag, diag);
    for (int j = 0; j < natoms; ++j) {
        const double zj = __shfl_sync(0xffffffffu, z, j);
        const double xj = __shfl_sync(0xffffffffu, x, j);
        const double yj = __shfl_sync(0xffffffffu, y, j);
        const double wj = __shfl_sync(0xffffffffu, w, j);
        if (!live) continue;
        double p;
        if (j == lane) {
            p = diag;
        } else {
            const double dx = __dsub_rn(xj, x);
            const double dy = __dsub_rn(yj, y);
            const double dz = __dsub_rn(wj, w);
            double s = __dmul_rn(dx, dx);
            s = __dadd_rn(s, __dmul_rn(dy, dy));
            s = __dadd_rn(s, __dmul_rn(dz, dz));
            p = __ddiv_rn(__dmul_rn(z, zj), __dsqrt_rn(s));
            norm = __dadd_rn(norm, __dmul_rn(p, p));
        }
        s_m[warp][lane][j] = p;
    }

    // Selection order.
    if (sorting) {
        double key = live ? norm : INFINITY;
        for (int k = 0; k < natoms; ++k) {
            double bv = key;
            int bi = lane;
            for (int off = 16; off > 0; off >>= 1) {
                const double ov = __shfl_xor_sync(0xffffffffu, bv, off);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                if (ov < bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            // Lanes beyond natoms hold +inf and never win while a live lane is
            // finite; a live lane whose norm is +inf (coincident atoms) behaves like
            // the reference: already-picked lanes (DBL_MAX) are picked again first.
            if (bi >= natoms) bi = 0;
            if (lane == 0) s_order[warp][natoms - 1 - k] = bi;
            if (lane == bi) key = DBL_MAX;
        }
    } else if (live) {
        s_order[warp][lane] = lane;
    }
    __syncwarp();

    // Packed lower triangle, then zero padding.
    const int filled = natoms * (natoms + 1) / 2;
    for (int e = lane; e < filled; e += 32) {
        // row m: largest m with m(m+1)/2 <= e
        int m = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
        while (m * (m + 1) / 2 > e) --m;
        while ((m + 1) * (m + 2) / 2 <= e) ++m;
        const int n = e - m * (m + 1) / 2;
        dst[e] = s_m[warp][s_order[warp][m]][s_order[warp][n]];
    }
    for (int64_t e = filled + lane; e < len; e += 32) dst[e] = 0.0;
}

std::once_flag g_table_once;
int g_table_status = QMLG_OK;

int upload_table()
{
    std::call_once(g_table_once, [] {
        double t[kZTable];
        for (int i = 0; i < kZTable; ++i) t[i] = std::pow((double)i, 2.4);
        cudaError_t e = cudaMemcpyToSymbol(c_zpow, t, sizeof(t));
        g_table_status = e == cudaSuccess ? QMLG_OK : qmlg::set_cuda_error(e);
    });
    return g_table_status;
}

}  // namespace

extern "C" int qmlg_coulomb_matrix(const double *charges, const double *coordinates,
                                   const int64_t *atom_offsets, int n_mol, int size,
                                   int sorting, double *out, int *status, void *stream)
{
    if (n_mol < 0 || size < 1) return QMLG_E_ARG;
    if (n_mol == 0) return QMLG_OK;
    if (atom_offsets == nullptr || out == nullptr) return QMLG_E_ARG;
    int st = upload_table();
    if (st != QMLG_OK) return st;
    const int blocks = (int)qmlg::ceil_div(n_mol, kWarpsPerBlock);
    { coulomb_kernel<<<blocks, kWarpsPerBlock * 32, 0, qmlg::as_stream(stream)>>>(
        charges, coordinates, atom_offsets, n_mol, size, sorting ? 1 : 0, out, status); qmlg::count_launches(1); }
    return qmlg::check_launch();
}
