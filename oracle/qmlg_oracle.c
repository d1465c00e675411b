/*
 * CPU oracle for the QML kernel-ridge-regression hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the reference's
 * Fortran routines for the molecular and atomic Coulomb matrices, the global and
 * local kernel matrices, plus a double-double residual used to refine solves.  Only the
 * tests, the smoke check and the CPU-baseline leg of the benchmark load it, as the
 * checker; the product path never calls it.
 *
 * Build with -ffp-contract=off: the restatement fixes one evaluation order (no
 * fused multiply-add contraction) so that the GPU kernels can reproduce the Coulomb
 * matrix bit for bit.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/*
 * Sorted Coulomb matrix of one molecule.
 * Follows qml/frepresentations.f90:52-140 (fgenerate_coulomb_matrix):
 *   M_ii = 0.5 * Z_i^2.4                                   (:95)
 *   M_ij = Z_i * Z_j / sqrt(sum_x (R_jx - R_ix)^2)         (:104-105)
 *   row norm_i = M_ii^2, then + M_ij^2 for j ascending, j != i (single-thread
 *   order of the reduction at :93-114)
 *   selection: natoms times, j = first index of the minimum row norm, placed at
 *   the end, its norm replaced by the largest double              (:116-121)
 *   packed lower triangle cm[m(m+1)/2 + n] = M[s_m, s_n], n <= m, rest zero
 *                                                                  (:124-134)
 * Returns 0, or -1 if natoms > nmax (the reference writes out of bounds there).
 */
int oracle_cm_sorted(const double *z, const double *r, int natoms, int nmax, double *cm)
{
    if (natoms > nmax || natoms < 0) return -1;
    const int len = nmax * (nmax + 1) / 2;
    memset(cm, 0, sizeof(double) * (size_t)len);
    if (natoms == 0) return 0;
    double *m = (double *)malloc(sizeof(double) * (size_t)natoms * (size_t)natoms);
    double *rn = (double *)malloc(sizeof(double) * (size_t)natoms);
    int *order = (int *)malloc(sizeof(int) * (size_t)natoms);
    for (int i = 0; i < natoms; ++i) {
        double p = 0.5 * pow(z[i], 2.4);
        m[i * natoms + i] = p;
    }
    for (int i = 0; i < natoms; ++i) {
        for (int j = i + 1; j < natoms; ++j) {
            double dx = r[3 * j + 0] - r[3 * i + 0];
            double dy = r[3 * j + 1] - r[3 * i + 1];
            double dz = r[3 * j + 2] - r[3 * i + 2];
            double s = dx * dx;
            s = s + dy * dy;
            s = s + dz * dz;
            double p = (z[i] * z[j]) / sqrt(s);
            m[i * natoms + j] = p;
            m[j * natoms + i] = p;
        }
    }
    for (int i = 0; i < natoms; ++i) {
        double d = m[i * natoms + i];
        double acc = d * d;
        for (int j = 0; j < natoms; ++j) {
            if (j == i) continue;
            double p = m[i * natoms + j];
            acc = acc + p * p;
        }
        rn[i] = acc;
    }
    for (int k = 0; k < natoms; ++k) {
        int best = 0;
        for (int j = 1; j < natoms; ++j)
            if (rn[j] < rn[best]) best = j;
        order[natoms - 1 - k] = best;
        rn[best] = DBL_MAX;
    }
    for (int a = 0; a < natoms; ++a) {
        const int base = a * (a + 1) / 2;
        for (int b = 0; b <= a; ++b) cm[base + b] = m[order[a] * natoms + order[b]];
    }
    free(m);
    free(rn);
    free(order);
    return 0;
}

/*
 * Unsorted Coulomb matrix: the same matrix in input order.
 * Follows qml/frepresentations.f90:142-205 (fgenerate_unsorted_coulomb_matrix).
 */
int oracle_cm_unsorted(const double *z, const double *r, int natoms, int nmax, double *cm)
{
    if (natoms > nmax || natoms < 0) return -1;
    const int len = nmax * (nmax + 1) / 2;
    memset(cm, 0, sizeof(double) * (size_t)len);
    for (int a = 0; a < natoms; ++a) {
        const int base = a * (a + 1) / 2;
        for (int b = 0; b < a; ++b) {
            double dx = r[3 * a + 0] - r[3 * b + 0];
            double dy = r[3 * a + 1] - r[3 * b + 1];
            double dz = r[3 * a + 2] - r[3 * b + 2];
            double s = dx * dx;
            s = s + dy * dy;
            s = s + dz * dz;
            cm[base + b] = (z[a] * z[b]) / sqrt(s);
        }
        cm[base + a] = 0.5 * pow(z[a], 2.4);
    }
    return 0;
}

/* Ragged batch: molecule m owns atoms offsets[m] .. offsets[m+1]-1. */
int oracle_cm_sorted_batch(const double *z, const double *r, const int64_t *offsets,
                           int n_mol, int nmax, double *out)
{
    const int len = nmax * (nmax + 1) / 2;
    int status = 0;
#pragma omp parallel for schedule(static) reduction(min : status)
    for (int mol = 0; mol < n_mol; ++mol) {
        const int64_t a = offsets[mol];
        const int n = (int)(offsets[mol + 1] - a);
        int st = oracle_cm_sorted(z + a, r + 3 * a, n, nmax, out + (size_t)mol * len);
        if (st < status) status = st;
    }
    return status;
}

/* cos(pi (d - cutoff + decay) / decay) + 1, pi = 4 atan(1): the reference applies
 * it as prefactor = 0.5d0 * (...) and as pair_norm = pair_norm * 0.5d0 * (...). */
static double cut_cos1(double d, double cutoff, double decay)
{
    const double pi = 4.0 * atan(1.0);
    return cos(pi * (d - cutoff + decay) / decay) + 1.0;
}

/*
 * Atomic (local) Coulomb matrices of one molecule, one row per central atom.
 * sorting 1 follows qml/frepresentations.f90:207-415 (fgenerate_local_coulomb_matrix,
 * "row-norm"), sorting 0 follows :417-595 (fgenerate_atomic_coulomb_matrix,
 * "distance"), single-thread loop order:
 *   cutoff adjustments (:254-271 / :457-474); D_ij = sqrt(sum_x (R_jx - R_ix)^2)
 *   for j > i; count_i = 1 + #{j != i: D_ij < central cutoff}; a central atom with
 *   count > nmax is an error (the reference stops).
 *   row-norm: per central atom k, for i ascending (skipped if D_ik > cc):
 *     pref = 1 or the central mask of D_ik; P_ii = pref pref 0.5 Z_i^2.4, rn_i += P_ii^2;
 *     for j > i (skipped if D_jk > cc or D_ij > ic): P_ij = pref Z_i Z_j / D_ij,
 *     times the interaction mask of D_ij and the central mask of D_jk where they
 *     apply; rn_i += P_ij^2, rn_j += P_ij^2.  rn_k = the largest double; count_k
 *     times j = first index of the maximum rn, rn_j = 0.
 *   distance: P_ii = 0.5 Z_i^2.4, P_ij = Z_i Z_j / D_ij (0 beyond ic, interaction
 *     mask); count_k times j = first index of the minimum of D_jk, replaced by the
 *     largest double; row m of the output (atom i = s_m) is skipped when D_ik > cc,
 *     else entry (m, n) = pref_i P_{s_m s_n} times the central mask of D_{s_n k}.
 *   packed lower triangle: out[m(m+1)/2 + n] for n <= m < count_k, rest zero.
 * central: ncentral atom indices (0-based).  out: ncentral x nmax(nmax+1)/2.
 * Returns 0, or -1 (bad arguments / too many atoms within the cutoff).
 */
int oracle_atomic_cm(const double *z, const double *r, int natoms, const int *central,
                     int ncentral, int nmax, int sorting, double cent_cutoff,
                     double cent_decay, double int_cutoff, double int_decay, double *out)
{
    const int len = nmax * (nmax + 1) / 2;
    if (natoms < 0 || ncentral < 0 || nmax < 1) return -1;
    memset(out, 0, sizeof(double) * (size_t)len * (size_t)ncentral);
    if (natoms == 0 || ncentral == 0) return 0;
    const double huge = DBL_MAX;
    if (cent_cutoff < 0) cent_cutoff = huge;
    if (int_cutoff < 0 || int_cutoff > 2 * cent_cutoff) int_cutoff = 2 * cent_cutoff;
    if (cent_decay < 0) cent_decay = 0.0;
    else if (cent_decay > cent_cutoff) cent_decay = cent_cutoff;
    if (int_decay < 0) int_decay = 0.0;
    else if (int_decay > int_cutoff) int_decay = int_cutoff;

    const size_t nn = (size_t)natoms * (size_t)natoms;
    double *D = (double *)calloc(nn, sizeof(double));
    double *P = (double *)calloc(nn, sizeof(double));
    double *rn = (double *)malloc(sizeof(double) * (size_t)natoms);
    double *dt = (double *)malloc(sizeof(double) * (size_t)natoms);
    int *cnt = (int *)malloc(sizeof(int) * (size_t)natoms);
    int *srt = (int *)malloc(sizeof(int) * (size_t)natoms);
    int status = 0;
    for (int i = 0; i < natoms; ++i) cnt[i] = 1;
    for (int i = 0; i < natoms; ++i)
        for (int j = i + 1; j < natoms; ++j) {
            double dx = r[3 * j + 0] - r[3 * i + 0];
            double dy = r[3 * j + 1] - r[3 * i + 1];
            double dz = r[3 * j + 2] - r[3 * i + 2];
            double s = dx * dx;
            s = s + dy * dy;
            s = s + dz * dz;
            const double nrm = sqrt(s);
            D[i * natoms + j] = nrm;
            D[j * natoms + i] = nrm;
            if (nrm < cent_cutoff) {
                cnt[i] += 1;
                cnt[j] += 1;
            }
        }
    for (int l = 0; l < ncentral; ++l)
        if (central[l] < 0 || central[l] >= natoms || cnt[central[l]] > nmax) status = -1;
    if (status == 0 && sorting == 0) {
        for (int i = 0; i < natoms; ++i) {
            P[i * natoms + i] = 0.5 * pow(z[i], 2.4);
            for (int j = i + 1; j < natoms; ++j) {
                const double dij = D[j * natoms + i];
                if (dij > int_cutoff) continue;
                double pn = z[i] * z[j] / dij;
                if (dij > int_cutoff - int_decay) pn = pn * 0.5 * cut_cos1(dij, int_cutoff, int_decay);
                P[i * natoms + j] = pn;
                P[j * natoms + i] = pn;
            }
        }
    }
    for (int l = 0; l < ncentral && status == 0; ++l) {
        const int k = central[l];
        double *o = out + (size_t)l * len;
        if (sorting == 1) {
            memset(P, 0, sizeof(double) * nn);
            for (int i = 0; i < natoms; ++i) rn[i] = 0.0;
            for (int i = 0; i < natoms; ++i) {
                const double dik = D[i * natoms + k];
                if (dik > cent_cutoff) continue;
                double pref = 1.0;
                if (dik > cent_cutoff - cent_decay) pref = 0.5 * cut_cos1(dik, cent_cutoff, cent_decay);
                double pn = pref * pref * 0.5 * pow(z[i], 2.4);
                P[i * natoms + i] = pn;
                rn[i] = rn[i] + pn * pn;
                for (int j = i + 1; j < natoms; ++j) {
                    const double djk = D[j * natoms + k], dij = D[i * natoms + j];
                    if (djk > cent_cutoff) continue;
                    if (dij > int_cutoff) continue;
                    pn = pref * z[i] * z[j] / D[j * natoms + i];
                    if (dij > int_cutoff - int_decay) pn = pn * 0.5 * cut_cos1(dij, int_cutoff, int_decay);
                    if (djk > cent_cutoff - cent_decay) pn = pn * 0.5 * cut_cos1(djk, cent_cutoff, cent_decay);
                    P[i * natoms + j] = pn;
                    P[j * natoms + i] = pn;
                    const double p2 = pn * pn;
                    rn[i] = rn[i] + p2;
                    rn[j] = rn[j] + p2;
                }
            }
            rn[k] = huge;
            for (int m = 0; m < cnt[k]; ++m) {
                int best = 0;
                for (int j = 1; j < natoms; ++j)
                    if (rn[j] > rn[best]) best = j;
                srt[m] = best;
                rn[best] = 0.0;
            }
            for (int m = 0; m < cnt[k]; ++m) {
                const int idx = (m * m + m) / 2;
                for (int n = 0; n <= m; ++n) o[idx + n] = P[srt[m] * natoms + srt[n]];
            }
        } else {
            for (int j = 0; j < natoms; ++j) dt[j] = D[j * natoms + k];
            for (int m = 0; m < cnt[k]; ++m) {
                int best = 0;
                for (int j = 1; j < natoms; ++j)
                    if (dt[j] < dt[best]) best = j;
                srt[m] = best;
                dt[best] = huge;
            }
            for (int m = 0; m < cnt[k]; ++m) {
                const int i = srt[m];
                const double dik = D[i * natoms + k];
                if (dik > cent_cutoff) continue;
                double pref = 1.0;
                if (dik > cent_cutoff - cent_decay) pref = 0.5 * cut_cos1(dik, cent_cutoff, cent_decay);
                const int idx = (m * m + m) / 2;
                for (int n = 0; n <= m; ++n) {
                    const int j = srt[n];
                    double pn = pref * P[i * natoms + j];
                    const double djk = D[j * natoms + k];
                    if (djk > cent_cutoff - cent_decay) pn = pn * 0.5 * cut_cos1(djk, cent_cutoff, cent_decay);
                    o[idx + n] = pn;
                }
            }
        }
    }
    free(D);
    free(P);
    free(rn);
    free(dt);
    free(cnt);
    free(srt);
    return status;
}

/*
 * Local kernels, kind 0 Gaussian (qml/fkernels.f90:23-108), 1 Laplacian (:110-196):
 * k[s + ns*(a + nm1*b)] = sum over atoms i of molecule a and j of molecule b of
 * exp(dist_ij * inv_s), dist = |q1_i - q2_j|^2 with inv_s = -0.5/sigma_s^2, or
 * dist = |q1_i - q2_j|_1 with inv_s = -1/sigma_s.  Atom rows are concatenated by
 * molecule (n1, n2: atom counts); the sum runs j-major over the (i, j) block like
 * Fortran's sum over atomic_distance(:ni, :nj).
 */
void oracle_local_kernels(int kind, const double *q1, const int *n1, int nm1, const double *q2,
                          const int *n2, int nm2, int d, const double *sigmas, int ns, double *k)
{
    int64_t *s1 = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nm1 + 1));
    int64_t *s2 = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nm2 + 1));
    double *inv = (double *)malloc(sizeof(double) * (size_t)(ns > 0 ? ns : 1));
    s1[0] = 0;
    for (int a = 0; a < nm1; ++a) s1[a + 1] = s1[a] + n1[a];
    s2[0] = 0;
    for (int b = 0; b < nm2; ++b) s2[b + 1] = s2[b] + n2[b];
    for (int t = 0; t < ns; ++t)
        inv[t] = kind == 0 ? -0.5 / (sigmas[t] * sigmas[t]) : -1.0 / sigmas[t];
#pragma omp parallel for schedule(dynamic)
    for (int a = 0; a < nm1; ++a) {
        for (int b = 0; b < nm2; ++b) {
            const int ni = n1[a], nj = n2[b];
            double *dm = (double *)malloc(sizeof(double) * (size_t)(ni > 0 ? ni : 1) * (size_t)(nj > 0 ? nj : 1));
            for (int i = 0; i < ni; ++i)
                for (int j = 0; j < nj; ++j) {
                    const double *x = q1 + (size_t)(s1[a] + i) * d, *y = q2 + (size_t)(s2[b] + j) * d;
                    double acc = 0.0;
                    for (int t = 0; t < d; ++t) {
                        const double u = x[t] - y[t];
                        acc = acc + (kind == 0 ? u * u : fabs(u));
                    }
                    dm[i + (size_t)ni * j] = acc;
                }
            for (int t = 0; t < ns; ++t) {
                double sum = 0.0;
                for (int j = 0; j < nj; ++j)
                    for (int i = 0; i < ni; ++i) sum = sum + exp(dm[i + (size_t)ni * j] * inv[t]);
                k[(size_t)t + (size_t)ns * ((size_t)a + (size_t)nm1 * b)] = sum;
            }
            free(dm);
        }
    }
    free(s1);
    free(s2);
    free(inv);
}

/*
 * Gaussian kernel matrix, Fortran order: k[j + i*na] = exp(-0.5/sigma^2 * |a_j - b_i|^2).
 * Follows qml/fkernels.f90:340-372 (fgaussian_kernel): direct difference form,
 * inv_sigma = -0.5/(sigma*sigma) (:357), sum over the feature index ascending.
 * a is na x d row-major (the Fortran d x na column-major view), b is nb x d.
 */
void oracle_gaussian_kernel(const double *a, int na, const double *b, int nb, int d,
                            double sigma, double *k)
{
    const double inv_sigma = -0.5 / (sigma * sigma);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nb; ++i) {
        const double *bi = b + (size_t)i * d;
        for (int j = 0; j < na; ++j) {
            const double *aj = a + (size_t)j * d;
            double s = 0.0;
            for (int t = 0; t < d; ++t) {
                double u = aj[t] - bi[t];
                s = s + u * u;
            }
            k[(size_t)j + (size_t)i * na] = exp(inv_sigma * s);
        }
    }
}

/*
 * Laplacian kernel matrix, Fortran order: k[j + i*na] = exp(-1/sigma * |a_j - b_i|_1).
 * Follows qml/fkernels.f90:374-400 (flaplacian_kernel), inv_sigma = -1/sigma (:390).
 */
void oracle_laplacian_kernel(const double *a, int na, const double *b, int nb, int d,
                             double sigma, double *k)
{
    const double inv_sigma = -1.0 / sigma;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nb; ++i) {
        const double *bi = b + (size_t)i * d;
        for (int j = 0; j < na; ++j) {
            const double *aj = a + (size_t)j * d;
            double s = 0.0;
            for (int t = 0; t < d; ++t) s = s + fabs(aj[t] - bi[t]);
            k[(size_t)j + (size_t)i * na] = exp(inv_sigma * s);
        }
    }
}

/*
 * Linear kernel, Fortran order: k[j + i*na] = dot(a_j, b_i).
 * Follows qml/fkernels.f90:403-423 (flinear_kernel): dot_product over the feature
 * index ascending.
 */
void oracle_linear_kernel(const double *a, int na, const double *b, int nb, int d, double *k)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nb; ++i) {
        const double *bi = b + (size_t)i * d;
        for (int j = 0; j < na; ++j) {
            const double *aj = a + (size_t)j * d;
            double s = 0.0;
            for (int t = 0; t < d; ++t) s = s + aj[t] * bi[t];
            k[(size_t)j + (size_t)i * na] = s;
        }
    }
}

/*
 * Matern kernel with the L2 distance, Fortran order.  Follows qml/fkernels.f90:426-484
 * (fmatern_kernel_l2): d2 = sum((a_j - b_i)^2), d = sqrt(d2);
 *   order 0: inv_sigma = -1/sigma,        k = exp(inv_sigma d)
 *   order 1: inv_sigma = -sqrt(3)/sigma,  k = exp(inv_sigma d) (1 - inv_sigma d)
 *   other:   inv_sigma = -sqrt(5)/sigma, inv_sigma2 = 5/(3 sigma^2),
 *            k = exp(inv_sigma d) (1 - inv_sigma d + inv_sigma2 d2)
 */
void oracle_matern_kernel_l2(const double *a, int na, const double *b, int nb, int d,
                             double sigma, int order, double *k)
{
    /* the reference's branches: order 0, order 1, anything else */
    const int form = order == 0 ? 0 : (order == 1 ? 1 : 2);
    double inv_sigma = -1.0 / sigma, inv_sigma2 = 0.0;
    if (form == 1) inv_sigma = -sqrt(3.0) / sigma;
    if (form == 2) {
        inv_sigma = -sqrt(5.0) / sigma;
        inv_sigma2 = 5.0 / (3.0 * sigma * sigma);
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nb; ++i) {
        const double *bi = b + (size_t)i * d;
        for (int j = 0; j < na; ++j) {
            const double *aj = a + (size_t)j * d;
            double d2 = 0.0;
            for (int t = 0; t < d; ++t) {
                double u = aj[t] - bi[t];
                d2 = d2 + u * u;
            }
            const double dd = sqrt(d2);
            double v = exp(inv_sigma * dd);
            if (form == 1) v = v * (1.0 - inv_sigma * dd);
            if (form == 2) v = v * (1.0 - inv_sigma * dd + inv_sigma2 * d2);
            k[(size_t)j + (size_t)i * na] = v;
        }
    }
}

/*
 * Sargan kernel, Fortran order.  Follows qml/fkernels.f90:487-531 (fsargan_kernel):
 * d = sum|a_j - b_i|, inv_sigma = -1/sigma,
 * k = exp(inv_sigma d) (1 + sum_m gammas[m-1] (-inv_sigma d)^m), m = 1..ng.
 */
void oracle_sargan_kernel(const double *a, int na, const double *b, int nb, int d, double sigma,
                          const double *gammas, int ng, double *k)
{
    const double inv_sigma = -1.0 / sigma;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < nb; ++i) {
        const double *bi = b + (size_t)i * d;
        for (int j = 0; j < na; ++j) {
            const double *aj = a + (size_t)j * d;
            double s = 0.0;
            for (int t = 0; t < d; ++t) s = s + fabs(aj[t] - bi[t]);
            double pre = 0.0, p = 1.0;
            for (int m = 0; m < ng; ++m) {
                p = p * (-inv_sigma * s);
                pre = pre + gammas[m] * p;
            }
            k[(size_t)j + (size_t)i * na] = exp(inv_sigma * s) * (1.0 + pre);
        }
    }
}

/* Error-free transformations (Knuth two-sum, fma two-product). */
static inline void two_sum(double a, double b, double *s, double *e)
{
    double x = a + b;
    double bv = x - a;
    double av = x - bv;
    *s = x;
    *e = (a - av) + (b - bv);
}

static inline void dd_add_prod(double *hi, double *lo, double a, double b)
{
    double p = a * b;
    double pe = fma(a, b, -p);
    double s, e;
    two_sum(*hi, p, &s, &e);
    e += pe + *lo;
    two_sum(s, e, hi, lo);
}

/*
 * r = y - (A + lambda I) x, with every product and sum carried in double-double,
 * rounded to double at the end.  A is n x n with leading dimension lda (symmetric:
 * row or column order gives the same result).  Used by the refined oracle solve.
 */
void oracle_residual_dd(const double *A, int n, int64_t lda, double lambda, const double *x,
                        const double *y, double *r)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
        const double *row = A + (size_t)i * (size_t)lda;
        double hi = y[i], lo = 0.0;
        for (int j = 0; j < n; ++j) dd_add_prod(&hi, &lo, -row[j], x[j]);
        dd_add_prod(&hi, &lo, -lambda, x[i]);
        r[i] = hi + lo;
    }
}

/*
 * r = y - A x for an m x n block of rows (leading dimension lda), every product and
 * sum carried in double-double and rounded to double at the end: the residual of a
 * sample of rows of a larger system, for backward-error checks at sizes where the
 * whole matrix is not copied to the host.
 */
void oracle_rows_residual_dd(const double *A, int m, int n, int64_t lda, const double *x,
                             const double *y, double *r)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < m; ++i) {
        const double *row = A + (size_t)i * (size_t)lda;
        double hi = y[i], lo = 0.0;
        for (int j = 0; j < n; ++j) dd_add_prod(&hi, &lo, -row[j], x[j]);
        r[i] = hi + lo;
    }
}
