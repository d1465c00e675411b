/*
 * CPU oracle for the QML kernel-ridge-regression hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C, the reference's
 * Fortran routines for the sorted Coulomb matrix and the Gaussian / Laplacian
 * kernel matrices, plus a double-double residual used to refine solves.  Only the
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
