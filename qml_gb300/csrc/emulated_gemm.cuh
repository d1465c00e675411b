// Emulated-FP64 products on the bf16 tensor cores (declarations).
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

// Trailing update C <- C - P P^T of the blocked Cholesky (rows/cols k0+nb .. n of the
// row-major lower triangle, P = the nb-wide panel at column k0), with P cut into
// `slices` digit planes.  digits: [slices][n][64] bf16, expo: [n] int (workspace).
int emu_trailing_update(double *A, int64_t lda, int n, int k0, int nb, int slices,
                        __nv_bfloat16 *digits, int *expo, const int *d_info, cudaStream_t s);

// In-place factor with emulated trailing updates; storage as the FP64 factor.
struct EmulatedFactor {
    double *A = nullptr;
    int n = 0;
    int64_t lda = 0;
    int slices = 0;
};

size_t emulated_factor_ws(int n);
int emulated_factor(double *A, int n, int64_t lda, double shift, Workspace &ws, int *d_info,
                    EmulatedFactor &f, cudaStream_t s, int slices = 8);
int emulated_potrs(const EmulatedFactor &f, double *x, cudaStream_t s);

// Shared with the FP64 path (cholesky.cu).
int cholesky_fp64(double *A, int n, int64_t lda, double shift, int *d_info, cudaStream_t s);
int potrs_fp64(const double *A, int n, int64_t lda, double *x, cudaStream_t s);
int mirror_upper_to_lower(double *A, int n, int64_t lda, const double *diag, cudaStream_t s);

}  // namespace qmlg
