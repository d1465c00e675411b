// Emulated-FP64 products on the bf16 tensor cores (declarations; kernels in
// emulated_tc.cu, the factorisation driver in cholesky.cu).
//
// GB300 runs FP64 at about 1.2 TFLOP/s, so FP64-accurate contractions are formed
// from exact integer products on the bf16 tensor cores instead (the splitting idea
// of Ozaki et al., "Error-free transformations of matrix multiplication by using
// fast routines of matrix multiplication", 2012, with fixed-point slices):
//   each FP64 row x_i is scaled by a power of two 2^-e_i so that |x| <= 1/2, then
//   cut into S signed base-128 digits d_s in [-64, 64] (exact in bf16):
//       x_i = 2^e_i * sum_s d_{i,s} 128^-(s+1)  (+ a remainder below 2^(e_i-7S-1));
//   digit products are integers below 2^12, so K-term sums of the digit planes
//   stay exact in FP32 accumulators (K*4096*pairs < 2^24); only the planes with
//   s + t <= S-1 are multiplied (the rest lies below the truncation);
//   the epilogue merges the levels in 64-bit integers and converts once to FP64.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace qmlg {

constexpr int kEmuMaxSlices = 8;

// Rows reserved per problem in a shared plane buffer, and the padded feature width.
inline int plane_rows(int n) { return (int)ceil_div(n < 1 ? 1 : n, 128) * 128; }
inline int plane_cols(int d) { return (int)ceil_div(d < 1 ? 1 : d, 64) * 64; }

// tcgen05 path (emulated_tc.cu).
// Digit planes of rows r0 .. r0+nrows-1, columns c0 .. c0+kw-1 of a row-major matrix:
// digits [slices][rpad][kp] bf16 (kp a multiple of 64, zero-padded), expo [rpad].
// norms (optional, [rpad]) receives the FP64 sum of squares of each row.
int slice_rows(const double *A, int64_t lda, int r0, int nrows, int c0, int kw, int kp, int rpad,
               int slices, __nv_bfloat16 *digits, int *expo, const int *d_info, cudaStream_t s,
               double *norms = nullptr);
// C[i][j] -= sum_k P[i][k] P[j][k] for j in [jbase, jend), i in [ibase, iend) (j <= i
// when lower), P rows taken from the digit planes (digit row = a_row0 + j - jbase for
// the j side, b_row0 + i - ibase for the i side), K = kp <= 512.
// max_ctas: 0 = the calling thread's default grid, > 0 = persistent grid of at most
// that many CTAs, < 0 = one CTA per tile.
int emu_tc_update(double *C, int64_t ldc, int jbase, int jend, int ibase, int iend,
                  const __nv_bfloat16 *digits, const int *expo, int kp, int rpad, int slices,
                  int a_row0, int b_row0, int lower, int *d_err, cudaStream_t s, int max_ctas = 0);
// SM count of the current device, after the calling thread's cap.
int tc_sm_count();

// Grouped launches: the tiles of many independent problems in one persistent launch
// (groups of up to 128 problems per launch).  Every problem's digit rows lie in one
// shared plane buffer: planes [slices][rows_total][kp] bf16, exponents [rows_total].
struct GroupItem {
    double *C;            // row-major C of the trailing update / column-major K
    int64_t ldc;
    int jbase, jend;      // lanes: contiguous index range of C
    int ibase, iend;      // TMEM columns
    int a_row0, b_row0;   // digit rows of j = jbase and i = ibase in the shared buffer
    double scale;         // Gaussian: -0.5 / sigma^2 (unused by the update)
};
// C_g[i][j] -= sum_k P[i][k] P[j][k] on the lower triangle (j <= i) of each item's
// range, K = kp <= 512 for all items.
// tile_cols: i-columns per tile, 64 (one TMEM accumulator) or 32 (two).
int emu_tc_group_update(const GroupItem *items, int count, const __nv_bfloat16 *digits,
                        const int *expo, int kp, int rows_total, int slices, int *d_err,
                        cudaStream_t s, int tile_cols = 64);

// Digit planes of many problems' row blocks in one launch, each into the shared plane
// buffer at its row0 (plane_rows(nrows) rows reserved): rows r0 .. r0+nrows-1,
// columns c0 .. c0+kw-1 of its row-major A, as slice_rows does.  info (may be null):
// nothing is done for a problem whose factorisation has failed.
struct SliceItem {
    const double *A;
    int64_t lda;
    int r0, nrows, c0, kw;
    int row0;
    const int *info;
};
int slice_rows_group(const SliceItem *items, int count, int kp, int rows_total, int slices,
                     __nv_bfloat16 *digits, int *expo, cudaStream_t s);

// Symmetric Gaussian kernel matrices of many problems, K = exp(-|x_i - x_j|^2 /
// (2 sigma^2)) in each problem's column-major K (ldk), K_ii = 1, with 8 digit planes:
// each problem's rows are sliced into the shared buffer at row0 (rows_pad(n) rows
// reserved; norms [rows_total] receive |x|^2), its 1e-12 bound is checked on the
// device (8 ORed into *flag when not met), then one grouped launch forms every K.
struct GaussItem {
    const double *X;
    int64_t ldx;
    int n;
    double sigma;
    double *K;
    int64_t ldk;
    int row0;
    int *flag;
};
int gauss_group_kernel_matrix(const GaussItem *items, int count, int d, __nv_bfloat16 *digits,
                              int *expo, double *norms, unsigned long long *maxbuf,
                              int rows_total, int *d_err, cudaStream_t s);


// In-place factor with emulated trailing updates; storage as the FP64 factor.
struct EmulatedFactor {
    double *A = nullptr;
    int n = 0;
    int64_t lda = 0;
    int slices = 0;
    int *d_err = nullptr;  // device flag: a bounded tensor-core wait gave up
    const double *Linv = nullptr;  // [n/64][64][64] inverses of the diagonal blocks
    const double *M = nullptr;     // [n/64][64][64] L_ii^-1 L_i,i-1 (the solves' couplings)
    const double *P = nullptr;     // [n/64][64][64] (L_i+1,i L_ii^-1)^T
    double *solved = nullptr;      // [2][n/64][64] solved entries of the two solves
};

size_t emulated_factor_ws(int n);
// npiv (a multiple of 64, or -1 for n): take only the first npiv pivots, leaving the
// Schur complement in the trailing block.
// coupled: as cholesky_fp64's (the inverse's augmented matrix).
int emulated_factor(double *A, int n, int64_t lda, double shift, Workspace &ws, int *d_info,
                    EmulatedFactor &f, cudaStream_t s, int slices = 8, int npiv = -1,
                    bool coupled = false);
int emulated_potrs(const EmulatedFactor &f, double *x, cudaStream_t s);
// A cooperative launch ordered after every earlier one of this process on the
// device (so two whole-GPU grids are never resident together), and whether one is
// allowed on the stream (not while capturing, not on threads that turned them off).
int launch_cooperative_serialised(const void *fn, int grid, int threads, void **args,
                                  cudaStream_t s);
bool cooperative_allowed_on(cudaStream_t s);
int read_device_flag(const int *d_flag, cudaStream_t s);

// Shared with the FP64 path (cholesky.cu).
// coupled: A is [[A_p, E], [E^T, 0]] with E = [I; 0] and npiv = A_p's size, so coupling
// row npiv + j is zero before pivot j and each panel only touches rows below
// npiv + (its last pivot + 1).
int cholesky_fp64(double *A, int n, int64_t lda, double shift, int *d_info, cudaStream_t s,
                  int npiv = -1, bool coupled = false);
int potrs_fp64(const double *A, int n, int64_t lda, double *x, cudaStream_t s);
int mirror_upper_to_lower(double *A, int n, int64_t lda, const double *diag, cudaStream_t s);

}  // namespace qmlg
