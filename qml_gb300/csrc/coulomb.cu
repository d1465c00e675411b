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
#include <climits>
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

    // M's pairs into shared memory, dealt out one per lane.  An FP64 instruction holds
    // its scheduler's FP64 pipe for the same time whatever its active lanes, so the
    // n(n-1)/2 pairs (i < j) go through the sqrt and division in n(n-1)/64 trips
    // instead of one trip per atom.  Pair (i, j) is what lane i formed before,
    // (z_i z_j) / sqrt(dx^2 + dy^2 + dz^2) with dx = x_j - x_i; lane j got the same
    // bits ((-dx)^2 = dx^2, z_j z_i = z_i z_j), so it is stored at (i, j) and (j, i).
    const int npairs = natoms * (natoms - 1) / 2;
    for (int t0 = 0; t0 < npairs; t0 += 32) {
        const int t = t0 + lane;
        const bool in = t < npairs;
        int i = 0, j = 1;
        if (in) {
            // t = j (j - 1) / 2 + i, 0 <= i < j
            j = (int)((1.0f + sqrtf(8.0f * (float)t + 1.0f)) * 0.5f);
            while (j * (j - 1) / 2 > t) --j;
            while ((j + 1) * j / 2 <= t) ++j;
            i = t - j * (j - 1) / 2;
        }
        const double zi_ = __shfl_sync(0xffffffffu, z, i), zj = __shfl_sync(0xffffffffu, z, j);
        const double xi = __shfl_sync(0xffffffffu, x, i), xj = __shfl_sync(0xffffffffu, x, j);
        const double yi = __shfl_sync(0xffffffffu, y, i), yj = __shfl_sync(0xffffffffu, y, j);
        const double wi = __shfl_sync(0xffffffffu, w, i), wj = __shfl_sync(0xffffffffu, w, j);
        if (in) {
            const double dx = __dsub_rn(xj, xi);
            const double dy = __dsub_rn(yj, yi);
            const double dz = __dsub_rn(wj, wi);
            double s = __dmul_rn(dx, dx);
            s = __dadd_rn(s, __dmul_rn(dy, dy));
            s = __dadd_rn(s, __dmul_rn(dz, dz));
            const double p = __ddiv_rn(__dmul_rn(zi_, zj), __dsqrt_rn(s));
            s_m[warp][i][j] = p;
            s_m[warp][j][i] = p;
        }
    }
    if (live) s_m[warp][lane][lane] = diag;
    __syncwarp();
    // row norm in the reference's order: the diagonal, then j ascending
    double norm = __dmul_rn(diag, diag);
    for (int j = 0; j < natoms; ++j) {
        if (!live || j == lane) continue;
        const double p = s_m[warp][lane][j];
        norm = __dadd_rn(norm, __dmul_rn(p, p));
    }

    // Selection order.
    if (sorting && __all_sync(0xffffffffu, !live || !(norm != norm))) {
        // no NaN norm: the norms (>= 0), DBL_MAX and +inf order as their bits do,
        // so the selection runs on integer keys (the same picks, ties included)
        long long key = live ? __double_as_longlong(norm) : __double_as_longlong(INFINITY);
        const long long picked = __double_as_longlong(DBL_MAX);
        for (int k = 0; k < natoms; ++k) {
            long long bv = key;
            int bi = lane;
            for (int off = 16; off > 0; off >>= 1) {
                const long long ov = __shfl_xor_sync(0xffffffffu, bv, off);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                if (ov < bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            if (bi >= natoms) bi = 0;
            if (lane == 0) s_order[warp][natoms - 1 - k] = bi;
            if (lane == bi) key = picked;
        }
    } else if (sorting) {
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

// ------------------------------------------------------------ atomic CM --
//
// Atomic (local) Coulomb matrices, one warp per central atom, restating
// fgenerate_local_coulomb_matrix ("row-norm", qml/frepresentations.f90:207-415) and
// fgenerate_atomic_coulomb_matrix ("distance", :417-595) in their single-thread
// arithmetic order, with no FMA contraction:
//   D_ij = sqrt((dx*dx + dy*dy) + dz*dz); count_i = 1 + #{j != i: D_ij < cc};
//   masks applied as pref = 0.5 (cos(pi (d - c + w)/w) + 1) and p = (p 0.5)(cos + 1);
//   row-norm: lane r adds its row norm's terms in the order the reference's loop
//     does (pairs (i, r), i < r; the diagonal; pairs (r, j), j > r), so the order
//     of the selection (first index of the maximum, the central atom first) is the
//     reference's; distance: first index of the minimum distance to the central atom.
// Lane i owns atom i (molecules of at most 32 atoms).  Bit-identical to the
// reference arithmetic where no cutoff mask applies (the default cutoffs); inside
// the mask the device cos can differ from the host's in the last bits.
constexpr int kAcmWarps = 2;

struct AcmParams {
    double cc, cd, ic, id;  // adjusted central / interaction cutoff and decay
    int size, sorting;
};

__device__ __forceinline__ double acm_cos1(double d, double c, double w)
{
    const double pi = 3.141592653589793;  // 4 atan(1) in FP64
    return __dadd_rn(cos(__ddiv_rn(__dmul_rn(pi, __dadd_rn(__dsub_rn(d, c), w)), w)), 1.0);
}

__device__ __forceinline__ double acm_pref(double dik, const AcmParams &q)
{
    return dik > q.cc - q.cd ? __dmul_rn(0.5, acm_cos1(dik, q.cc, q.cd)) : 1.0;
}

typedef double AcmRow[kMaxAtoms + 1];

// One central atom (task) of molecule mol by the reference's per-centre steps, on
// one warp with its shared arrays D (distances), P (pair values) and ord.
__device__ void acm_task(const double *__restrict__ charges, const double *__restrict__ coords,
                         const int64_t *__restrict__ offsets, const int64_t *__restrict__ coff,
                         const int *__restrict__ central, int task, int mol, const AcmParams &q,
                         double *__restrict__ out, int *__restrict__ status, AcmRow *D, AcmRow *P,
                         int *ord)
{
    const int lane = threadIdx.x & 31;
    const int64_t len = (int64_t)q.size * (q.size + 1) / 2;
    double *dst = out + (int64_t)task * len;
    const int64_t first = offsets[mol];
    const int natoms = (int)(offsets[mol + 1] - first);
    const int k = central != nullptr ? central[task] : (int)(task - coff[mol]);
    for (int64_t e = lane; e < len; e += 32) dst[e] = 0.0;
    if (natoms > kMaxAtoms || natoms < 1 || k < 0 || k >= natoms) {
        if (lane == 0 && status != nullptr) atomicMin(status, natoms > kMaxAtoms ? QMLG_E_TOO_MANY_ATOMS : QMLG_E_ARG);
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
    double zp = 0.0;
    const int zi = (int)z;
    if ((double)zi == z && zi >= 0 && zi < kZTable) zp = c_zpow[zi];
    else zp = pow(z, 2.4);
    // distances and cutoff counts
    int cnt = 1;
    for (int j = 0; j < natoms; ++j) {
        const double xj = __shfl_sync(0xffffffffu, x, j);
        const double yj = __shfl_sync(0xffffffffu, y, j);
        const double wj = __shfl_sync(0xffffffffu, w, j);
        if (!live) continue;
        double dd = 0.0;
        if (j != lane) {
            const double dx = __dsub_rn(xj, x), dy = __dsub_rn(yj, y), dz = __dsub_rn(wj, w);
            double s2 = __dmul_rn(dx, dx);
            s2 = __dadd_rn(s2, __dmul_rn(dy, dy));
            s2 = __dadd_rn(s2, __dmul_rn(dz, dz));
            dd = __dsqrt_rn(s2);
            if (dd < q.cc) ++cnt;
        }
        D[lane][j] = dd;
    }
    __syncwarp();
    const int cntk = __shfl_sync(0xffffffffu, cnt, k);
    if (cntk > q.size) {
        if (lane == 0 && status != nullptr) atomicMin(status, QMLG_E_TOO_MANY_ATOMS);
        return;
    }
    const double dk = live ? D[lane][k] : 0.0;  // this atom's distance to the centre
    if (q.sorting == 1) {
        // pair value P(a, b), a < b, as the reference's loop forms it (0 when skipped)
        auto pair = [&](int a, int b, double za, double zb) -> double {
            const double dak = D[a][k], dbk = D[b][k], dab = D[a][b];
            if (dak > q.cc || dbk > q.cc || dab > q.ic) return 0.0;
            double pn = __ddiv_rn(__dmul_rn(__dmul_rn(acm_pref(dak, q), za), zb), D[b][a]);
            if (dab > q.ic - q.id) pn = __dmul_rn(__dmul_rn(pn, 0.5), acm_cos1(dab, q.ic, q.id));
            if (dbk > q.cc - q.cd) pn = __dmul_rn(__dmul_rn(pn, 0.5), acm_cos1(dbk, q.cc, q.cd));
            return pn;
        };
        double rn = 0.0;
        for (int i = 0; i < natoms; ++i) {
            const double zo = __shfl_sync(0xffffffffu, z, i);
            if (!live) continue;
            double p;
            if (i < lane) {
                p = pair(i, lane, zo, z);
                if (D[i][k] <= q.cc && dk <= q.cc && D[i][lane] <= q.ic)
                    rn = __dadd_rn(rn, __dmul_rn(p, p));
            } else if (i == lane) {
                p = 0.0;
                if (dk <= q.cc) {
                    const double pr = acm_pref(dk, q);
                    p = __dmul_rn(__dmul_rn(__dmul_rn(pr, pr), 0.5), zp);
                    rn = __dadd_rn(rn, __dmul_rn(p, p));
                }
            } else {
                p = pair(lane, i, z, zo);
                if (dk <= q.cc && D[i][k] <= q.cc && D[lane][i] <= q.ic)
                    rn = __dadd_rn(rn, __dmul_rn(p, p));
            }
            P[lane][i] = p;
        }
        double key = live ? (lane == k ? DBL_MAX : rn) : -INFINITY;
        for (int m = 0; m < cntk; ++m) {
            double bv = key;
            int bi = lane;
            for (int off = 16; off > 0; off >>= 1) {
                const double ov = __shfl_xor_sync(0xffffffffu, bv, off);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                if (ov > bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            if (lane == 0) ord[m] = bi;
            if (lane == bi) key = 0.0;
        }
        __syncwarp();
        for (int m = 0; m < cntk; ++m) {
            const int idx = (m * m + m) / 2, a = ord[m];
            for (int n = lane; n <= m; n += 32) dst[idx + n] = P[a][ord[n]];
        }
    } else {
        // centre-independent pair matrix
        for (int j = 0; j < natoms; ++j) {
            const double zo = __shfl_sync(0xffffffffu, z, j);
            if (!live) continue;
            double p;
            if (j == lane) {
                p = __dmul_rn(0.5, zp);
            } else {
                const double dij = D[lane][j];
                p = 0.0;
                if (!(dij > q.ic)) {
                    const double za = j < lane ? zo : z, zb = j < lane ? z : zo;
                    p = __ddiv_rn(__dmul_rn(za, zb), dij);
                    if (dij > q.ic - q.id) p = __dmul_rn(__dmul_rn(p, 0.5), acm_cos1(dij, q.ic, q.id));
                }
            }
            P[lane][j] = p;
        }
        double key = live ? dk : INFINITY;
        for (int m = 0; m < cntk; ++m) {
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
            if (lane == 0) ord[m] = bi;
            if (lane == bi) key = DBL_MAX;
        }
        __syncwarp();
        for (int m = 0; m < cntk; ++m) {
            const int i = ord[m];
            const double dik = D[i][k];
            if (dik > q.cc) continue;
            const double pr = acm_pref(dik, q);
            const int idx = (m * m + m) / 2;
            for (int n = lane; n <= m; n += 32) {
                const int j = ord[n];
                double pn = __dmul_rn(pr, P[i][j]);
                const double djk = D[j][k];
                if (djk > q.cc - q.cd) pn = __dmul_rn(__dmul_rn(pn, 0.5), acm_cos1(djk, q.cc, q.cd));
                dst[idx + n] = pn;
            }
        }
    }
}


// Order-preserving integer key of a double >= 0.
__device__ __forceinline__ long long acm_key(double v) { return __double_as_longlong(v); }

// One warp per molecule.  Where no cutoff or decay mask touches the molecule (every
// distance positive, inside the central cutoff and below both decay bands: the
// default cutoffs), the prefactors are all 1.0, so the pair values, and for row-norm
// sorting the row norms, are the same for every central atom: the warp forms them
// once and writes every centre's row from them, with the arithmetic acm_task uses
// (multiplying by a prefactor of 1.0 is exact), so the rows are the same bits.
// Row-norm order for centre k is k, then the molecule's one descending order
// without k; distance order is selected per centre on integer keys.  Any other
// molecule runs acm_task for each of its central atoms.
__global__ void __launch_bounds__(kAcmWarps * 32)
atomic_cm_kernel(const double *__restrict__ charges, const double *__restrict__ coords,
                 const int64_t *__restrict__ offsets, int n_mol,
                 const int64_t *__restrict__ central_offsets, const int *__restrict__ central,
                 int n_central, AcmParams q, double *__restrict__ out, int *__restrict__ status)
{
    __shared__ double sD[kAcmWarps][kMaxAtoms][kMaxAtoms + 1];
    __shared__ double sP[kAcmWarps][kMaxAtoms][kMaxAtoms + 1];
    __shared__ int sOrd[kAcmWarps][kMaxAtoms];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mol = blockIdx.x * kAcmWarps + warp;
    if (mol >= n_mol) return;
    const int64_t *coff = central_offsets != nullptr ? central_offsets : offsets;
    const int64_t t0 = coff[mol], t1 = coff[mol + 1];
    if (t0 >= t1 || t0 >= n_central) return;
    const int64_t first = offsets[mol];
    const int natoms = (int)(offsets[mol + 1] - first);
    const int64_t len = (int64_t)q.size * (q.size + 1) / 2;
    bool fast = natoms >= 1 && natoms <= kMaxAtoms && natoms <= q.size && t1 <= n_central;
    if (fast) {
        bool kok = true;
        for (int64_t t = t0 + lane; t < t1; t += 32) {
            const int k = central != nullptr ? central[t] : (int)(t - t0);
            kok = kok && k >= 0 && k < natoms;
        }
        fast = __all_sync(0xffffffffu, kok);
    }
    const bool live = lane < natoms;
    double z = 0.0, zp = 0.0, rn = 0.0;
    if (fast) {
        double x = 0.0, y = 0.0, w = 0.0;
        if (live) {
            z = charges[first + lane];
            x = coords[3 * (first + lane) + 0];
            y = coords[3 * (first + lane) + 1];
            w = coords[3 * (first + lane) + 2];
        }
        const int zi = (int)z;
        if ((double)zi == z && zi >= 0 && zi < kZTable) zp = c_zpow[zi];
        else zp = pow(z, 2.4);
        bool ok = true;
        for (int j = 0; j < natoms; ++j) {
            const double xj = __shfl_sync(0xffffffffu, x, j);
            const double yj = __shfl_sync(0xffffffffu, y, j);
            const double wj = __shfl_sync(0xffffffffu, w, j);
            if (!live) continue;
            double dd = 0.0;
            if (j != lane) {
                const double dx = __dsub_rn(xj, x), dy = __dsub_rn(yj, y), dz = __dsub_rn(wj, w);
                double s2 = __dmul_rn(dx, dx);
                s2 = __dadd_rn(s2, __dmul_rn(dy, dy));
                s2 = __dadd_rn(s2, __dmul_rn(dz, dz));
                dd = __dsqrt_rn(s2);
                ok = ok && dd > 0.0 && dd < q.cc && dd <= q.cc - q.cd && dd <= q.ic - q.id &&
                     dd <= q.ic;
            }
            sD[warp][lane][j] = dd;
        }
        fast = __all_sync(0xffffffffu, ok);
    }
    if (fast) {
        __syncwarp();
        // pair values: 0.5 Z^2.4 on the diagonal, Z_a Z_b / D_ab (a the smaller index)
        for (int j = 0; j < natoms; ++j) {
            const double zo = __shfl_sync(0xffffffffu, z, j);
            if (!live) continue;
            double p;
            if (j == lane) {
                p = __dmul_rn(0.5, zp);
            } else {
                const double za = j < lane ? zo : z, zb = j < lane ? z : zo;
                p = __ddiv_rn(__dmul_rn(za, zb), sD[warp][lane][j]);
            }
            sP[warp][lane][j] = p;
            rn = __dadd_rn(rn, __dmul_rn(p, p));
        }
        __syncwarp();
        // the selections below need every row norm positive and below DBL_MAX
        if (q.sorting == 1) fast = __all_sync(0xffffffffu, !live || (rn > 0.0 && rn < DBL_MAX));
    }
    if (!fast) {
        for (int64_t t = t0; t < t1 && t < n_central; ++t) {
            __syncwarp();
            acm_task(charges, coords, offsets, coff, central, (int)t, mol, q, out, status,
                     sD[warp], sP[warp], sOrd[warp]);
        }
        return;
    }
    int posk_base = 0;
    if (q.sorting == 1) {
        // the molecule's order: row norm descending, the first index among equals
        long long key = live ? acm_key(rn) : -1ll;
        for (int m = 0; m < natoms; ++m) {
            long long bv = key;
            int bi = lane;
            for (int off = 16; off > 0; off >>= 1) {
                const long long ov = __shfl_xor_sync(0xffffffffu, bv, off);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                if (ov > bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            if (lane == 0) sOrd[warp][m] = bi;
            if (lane == bi) {
                key = -2ll;
                posk_base = m;  // this lane's place in the order
            }
        }
        __syncwarp();
    }
    const int tri = natoms * (natoms + 1) / 2;
    for (int64_t t = t0; t < t1; ++t) {
        const int k = central != nullptr ? central[t] : (int)(t - t0);
        double *dst = out + t * len;
        for (int64_t e = tri + lane; e < len; e += 32) dst[e] = 0.0;
        int ordl = 0;  // lane m < natoms: the atom in place m for this centre
        if (q.sorting == 1) {
            const int pk = __shfl_sync(0xffffffffu, posk_base, k);
            if (live) ordl = lane == 0 ? k : sOrd[warp][lane - 1 < pk ? lane - 1 : lane];
        } else {
            // distance to the centre ascending, the first index among equals
            long long key = live ? acm_key(sD[warp][lane][k]) : LLONG_MAX;
            for (int m = 0; m < natoms; ++m) {
                long long bv = key;
                int bi = lane;
                for (int off = 16; off > 0; off >>= 1) {
                    const long long ov = __shfl_xor_sync(0xffffffffu, bv, off);
                    const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
                    if (ov < bv || (ov == bv && oi < bi)) {
                        bv = ov;
                        bi = oi;
                    }
                }
                if (lane == m) ordl = bi;
                if (lane == bi) key = LLONG_MAX - 1;
            }
        }
        // entry e of the packed lower triangle: row m, column n <= m (every lane runs
        // every trip, so the shuffles see the whole warp)
        int m = 0;
        for (int e0 = 0; e0 < tri; e0 += 32) {
            const int e = e0 + lane;
            const bool in = e < tri;
            if (in)
                while ((m + 1) * (m + 2) / 2 <= e) ++m;
            const int n = in ? e - m * (m + 1) / 2 : 0;
            const int a = __shfl_sync(0xffffffffu, ordl, in ? m : 0);
            const int b2 = __shfl_sync(0xffffffffu, ordl, n);
            if (in) dst[e] = sP[warp][a][b2];
        }
    }
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

extern "C" int qmlg_atomic_coulomb_matrix(const double *charges, const double *coordinates,
                                          const int64_t *atom_offsets, int n_mol,
                                          const int64_t *central_offsets, const int *central_atoms,
                                          int n_central, int size, int sorting,
                                          double central_cutoff, double central_decay,
                                          double interaction_cutoff, double interaction_decay,
                                          double *out, int *status, void *stream)
{
    if (n_mol < 0 || n_central < 0 || size < 1 || (sorting != 0 && sorting != 1)) return QMLG_E_ARG;
    if (n_mol == 0 || n_central == 0) return QMLG_OK;
    if (atom_offsets == nullptr || out == nullptr || charges == nullptr || coordinates == nullptr)
        return QMLG_E_ARG;
    if ((central_offsets == nullptr) != (central_atoms == nullptr)) return QMLG_E_ARG;
    int st = upload_table();
    if (st != QMLG_OK) return st;
    // the reference's cutoff adjustments (qml/frepresentations.f90:254-271)
    AcmParams q;
    const double huge = DBL_MAX;
    q.cc = central_cutoff < 0 ? huge : central_cutoff;
    q.ic = (interaction_cutoff < 0 || interaction_cutoff > 2 * q.cc) ? 2 * q.cc : interaction_cutoff;
    q.cd = central_decay < 0 ? 0.0 : (central_decay > q.cc ? q.cc : central_decay);
    q.id = interaction_decay < 0 ? 0.0 : (interaction_decay > q.ic ? q.ic : interaction_decay);
    q.size = size;
    q.sorting = sorting;
    const int blocks = (int)qmlg::ceil_div(n_mol, kAcmWarps);
    {
        atomic_cm_kernel<<<blocks, kAcmWarps * 32, 0, qmlg::as_stream(stream)>>>(
            charges, coordinates, atom_offsets, n_mol, central_offsets, central_atoms, n_central, q,
            out, status);
        qmlg::count_launches(1);
    }
    return qmlg::check_launch();
}
