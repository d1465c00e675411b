/*
 * qmlg: GB300-native (sm_103a) kernel-ridge-regression hot path for QML.
 *
 * C ABI of libqmlg.so.  Every entry point:
 *   - takes DEVICE pointers owned by the caller (for example torch tensors) and a
 *     cudaStream_t passed as void*; work is enqueued on that stream;
 *   - allocates nothing: scratch comes from a caller workspace whose size the
 *     matching *_workspace_size() call returns;
 *   - returns an int status: 0 = ok, > 0 = numerical information (for the
 *     Cholesky, the 1-based order of the first non-positive leading minor, like
 *     LAPACK's info), < 0 = argument or CUDA error (QMLG_E_* below).
 *
 * Matrices follow the reference's Fortran conventions: a kernel matrix K(na, nb)
 * is column-major with leading dimension ldk (K[j + i*ldk] = k(A_j, B_i)), and a
 * representation block A(na, d) is row-major with leading dimension lda (the
 * d x na column-major array the Fortran routines receive).
 */
#ifndef QMLG_H
#define QMLG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QMLG_OK 0
#define QMLG_E_ARG (-1)        /* bad size, stride, pointer or flag */
#define QMLG_E_CUDA (-2)       /* a CUDA launch or runtime call failed */
#define QMLG_E_WORKSPACE (-3)  /* workspace missing or too small */
#define QMLG_E_TOO_MANY_ATOMS (-4) /* a molecule has more atoms than size (or than 32) */
#define QMLG_E_NOT_CONVERGED (-5)  /* refinement did not reach its tolerance */
#define QMLG_E_TIMEOUT (-6)    /* a bounded device-side wait gave up */
#define QMLG_E_TOO_LARGE (-7)  /* problem exceeds a fixed-size internal buffer */

/* ---- library ---------------------------------------------------------- */

/* Version string and the compute capability the library was built for. */
const char *qmlg_version(void);

/* Last CUDA error string seen by the library on this host thread ("" if none). */
const char *qmlg_last_error(void);

/* Number of CUDA kernels this library has launched in this process so far. */
uint64_t qmlg_launch_count(void);

/*
 * Caps the grid of the persistent and cooperative kernels launched from the
 * calling host thread at n CTAs (0 = no cap, the default).  A serving process
 * gives its fit thread a cap so that query kernels on other streams always find
 * free SMs instead of waiting behind a whole-GPU factorisation.
 */
void qmlg_set_thread_sm_limit(int n);

/*
 * on = 1 (default): tensor-core kernels launched from the calling host thread use
 * persistent CTAs (one per SM, looping over tiles, loads of the next tile
 * overlapping the current epilogue).  on = 0: one CTA per tile, so a launch that
 * shares the GPU with other work spreads over whichever SMs are free; serving
 * threads use this for query kernels.
 */
void qmlg_set_thread_persistent(int on);

/*
 * on = 1 (default): the triangular solves of the Cholesky solve run as
 * cooperative grid-synchronised kernels over every SM (one at a time on the
 * device; the library chains them with an event).  on = 0: single-CTA solves with
 * the diagonal-block inverses, which any number of concurrent solves may run side
 * by side; batched work uses this.  Stream capture always takes the single-CTA
 * path.
 */
void qmlg_set_thread_cooperative(int on);

/* ---- sorted Coulomb matrix --------------------------------------------- */

/*
 * Row-norm sorted Coulomb matrix of a ragged batch of molecules.
 * Replaces fgenerate_coulomb_matrix (qml/frepresentations.f90:52-140), bound by
 * qml.representations.generate_coulomb_matrix (qml/representations.py:69-111),
 * which handles one molecule per call.
 *   charges      [total_atoms]      nuclear charges (FP64, like f2py's cast)
 *   coordinates  [total_atoms * 3]  x, y, z per atom
 *   atom_offsets [n_mol + 1]        molecule m owns atoms offsets[m] .. offsets[m+1]-1
 *   out          [n_mol * size*(size+1)/2]  packed lower triangle per molecule
 *   sorting      1 = row-norm sorted (the reference's "row-norm"),
 *                0 = input order ("unsorted", frepresentations.f90:142-205)
 *   status       [1] device int, set to QMLG_E_TOO_MANY_ATOMS if any molecule
 *                has more than size (or 32) atoms; may be NULL
 * The permutation and every value match the reference arithmetic bit for bit
 * (no FMA contraction; Z^2.4 from a host table for integer charges 0..127).
 */
int qmlg_coulomb_matrix(const double *charges, const double *coordinates,
                        const int64_t *atom_offsets, int n_mol, int size, int sorting,
                        double *out, int *status, void *stream);

/*
 * Atomic (local) Coulomb matrices: one row of size*(size+1)/2 per central atom.
 * Replaces fgenerate_local_coulomb_matrix (sorting 1, "row-norm",
 * qml/frepresentations.f90:207-415) and fgenerate_atomic_coulomb_matrix (sorting
 * 0, "distance", :417-595), bound by
 * qml.representations.generate_atomic_coulomb_matrix (qml/representations.py:121-230),
 * which handles one molecule per call.
 *   atom_offsets    [n_mol + 1]  molecule m owns atoms offsets[m] .. offsets[m+1]-1
 *   central_offsets [n_mol + 1], central_atoms [n_central]: the central atoms of
 *                   molecule m (indices within the molecule) are
 *                   central_atoms[central_offsets[m] .. central_offsets[m+1]-1];
 *                   both NULL: every atom is central (n_central = total atoms)
 *   out             [n_central * size*(size+1)/2], rows in central-atom order
 *   cutoffs/decays  as the reference: negative = none; adjusted like :254-271
 *   status          [1] device int: QMLG_E_TOO_MANY_ATOMS if a molecule has more
 *                   than 32 atoms or more than `size` atoms within the central
 *                   cutoff (the reference stops there), QMLG_E_ARG for a bad
 *                   central index; may be NULL
 * Where no cutoff mask applies the values and the atom order are the reference's
 * arithmetic bit for bit (no FMA contraction, Z^2.4 from the host table).
 */
int qmlg_atomic_coulomb_matrix(const double *charges, const double *coordinates,
                               const int64_t *atom_offsets, int n_mol,
                               const int64_t *central_offsets, const int *central_atoms,
                               int n_central, int size, int sorting, double central_cutoff,
                               double central_decay, double interaction_cutoff,
                               double interaction_decay, double *out, int *status, void *stream);

/* ---- kernel matrices ----------------------------------------------------- */

#define QMLG_KERNEL_SYMMETRIC 1   /* A == B: compute one triangle, mirror it */

/*
 * Gaussian kernel K(na, nb), K[j + i*ldk] = exp(-0.5/sigma^2 * |A_j - B_i|^2).
 * Replaces fgaussian_kernel (qml/fkernels.f90:340-372), bound by
 * qml.kernels.gaussian_kernel (qml/kernels.py:65-92).  FP64 arithmetic.
 * flags: QMLG_KERNEL_SYMMETRIC requires A == B and na == nb.
 * diag_shift is added to K[j + j*ldk] in symmetric mode (the KRR lambda); pass 0
 * for the reference's behaviour.
 */
int qmlg_gaussian_kernel(const double *A, int64_t lda, int na, const double *B, int64_t ldb,
                         int nb, int d, double sigma, double *K, int64_t ldk, int flags,
                         double diag_shift, void *stream);

/*
 * Laplacian kernel K(na, nb), K[j + i*ldk] = exp(-1/sigma * |A_j - B_i|_1).
 * Replaces flaplacian_kernel (qml/fkernels.f90:374-400), bound by
 * qml.kernels.laplacian_kernel (qml/kernels.py:36-63).  FP64 arithmetic.
 */
int qmlg_laplacian_kernel(const double *A, int64_t lda, int na, const double *B, int64_t ldb,
                          int nb, int d, double sigma, double *K, int64_t ldk, int flags,
                          double diag_shift, void *stream);

/*
 * Linear kernel K(na, nb), K[j + i*ldk] = A_j . B_i.  Replaces flinear_kernel
 * (qml/fkernels.f90:403-423), bound by qml.kernels.linear_kernel
 * (qml/kernels.py:94-120).  FP64 arithmetic; flags and diag_shift as above.
 */
int qmlg_linear_kernel(const double *A, int64_t lda, int na, const double *B, int64_t ldb, int nb,
                       int d, double *K, int64_t ldk, int flags, double diag_shift, void *stream);

/*
 * Matern kernel with the L2 distance d = |A_j - B_i|_2, order 0, 1 or 2:
 *   0: exp(-d/sigma)
 *   1: exp(-sqrt3 d/sigma) (1 + sqrt3 d/sigma)
 *   2: exp(-sqrt5 d/sigma) (1 + sqrt5 d/sigma + 5 d^2 / (3 sigma^2))
 * Replaces fmatern_kernel_l2 (qml/fkernels.f90:426-484), bound by
 * qml.kernels.matern_kernel(metric="l2") (qml/kernels.py:158-215); the L1 metric is
 * the Sargan kernel below, as the reference's wrapper maps it.  FP64 arithmetic.
 */
int qmlg_matern_kernel_l2(const double *A, int64_t lda, int na, const double *B, int64_t ldb,
                          int nb, int d, double sigma, int order, double *K, int64_t ldk,
                          int flags, double diag_shift, void *stream);

/*
 * Sargan kernel with the L1 distance d = |A_j - B_i|_1:
 *   exp(-d/sigma) (1 + sum_{m=1..ngammas} gammas[m-1] (d/sigma)^m).
 * gammas: device array of ngammas doubles (may be NULL when ngammas = 0, which gives
 * the Laplacian kernel).  Replaces fsargan_kernel (qml/fkernels.f90:487-531), bound
 * by qml.kernels.sargan_kernel (qml/kernels.py:122-156).  FP64 arithmetic.
 */
int qmlg_sargan_kernel(const double *A, int64_t lda, int na, const double *B, int64_t ldb, int nb,
                       int d, double sigma, const double *gammas, int ngammas, double *K,
                       int64_t ldk, int flags, double diag_shift, void *stream);

/*
 * Local (atomic) kernels, kind 0 Gaussian / 1 Laplacian, for several sigmas:
 *   K[s + nsigmas*(a + nm1*b)] = sum_{i in molecule a} sum_{j in molecule b}
 *                                exp(-|A_i - B_j|_2^2 / (2 sigma_s^2))  (Gaussian)
 *                                exp(-|A_i - B_j|_1 / sigma_s)          (Laplacian)
 * A, B: atom rows (lda, ldb >= d) grouped by molecule through offsets_a [nm1 + 1]
 * and offsets_b [nm2 + 1]; sigmas: device array; K: nsigmas x nm1 x nm2 with sigma
 * fastest (the reference's Fortran-ordered (nsigmas, nm1, nm2)).  Replaces
 * fget_local_kernels_gaussian / _laplacian (qml/fkernels.f90:23-196), bound by
 * qml.kernels.get_local_kernels_* (qml/kernels.py:218-299).  FP64 arithmetic.
 * flags: QMLG_KERNEL_SYMMETRIC (A == B, same offsets) computes b >= a and mirrors.
 */
int qmlg_local_kernels(int kind, const double *A, int64_t lda, const int64_t *offsets_a, int nm1,
                       const double *B, int64_t ldb, const int64_t *offsets_b, int nm2, int d,
                       const double *sigmas, int nsigmas, double *K, int flags, void *stream);

/*
 * The same local kernels from atom-pair kernel matrices: for each sigma and each
 * chunk of A's molecules (about 2 GiB of atom pairs), qmlg_gaussian_kernel_emulated
 * (tensor cores) or qmlg_laplacian_kernel_fixed (fixed-point L1 sums) gives the
 * chunk's atoms against all of B's, then two reductions sum them per molecule pair.
 * Every term is positive, so each entry keeps the atom-pair kernel's relative bound
 * (1e-12; those calls take their FP64 kernels where the bound cannot be met).
 * Arguments as qmlg_local_kernels, with both offset arrays starting at 0
 * (QMLG_E_ARG otherwise).  Reads the offsets and sigmas back to the host first (a
 * synchronisation).  QMLG_E_TOO_LARGE when one molecule holds more atoms
 * than a chunk's rows.  ws: qmlg_local_kernels_emulated_workspace_size(kind,
 * atoms of A, atoms of B, nm2, d).
 */
size_t qmlg_local_kernels_emulated_workspace_size(int kind, int64_t natoms_a, int64_t natoms_b,
                                                  int nm2, int d);
int qmlg_local_kernels_emulated(int kind, const double *A, int64_t lda, const int64_t *offsets_a,
                                int nm1, const double *B, int64_t ldb, const int64_t *offsets_b,
                                int nm2, int d, const double *sigmas, int nsigmas, double *K,
                                int flags, void *workspace, size_t ws_bytes, void *stream);

/*
 * Gaussian kernel with the contraction a.b emulated to FP64 accuracy on the bf16
 * tensor cores (tcgen05): rows are scaled by powers of two and cut into base-128
 * digit planes; the digit products are summed exactly in tensor memory and
 * merged, |a|^2 + |b|^2 - 2 a.b and exp are evaluated in FP64 in the epilogue.
 * The number of digit planes is chosen from a worst-case bound so that every
 * entry stays within 1e-12 relative of the FP64 kernel; when no plane count up to
 * 8 reaches it (very small sigma) the FP64 kernel above runs instead.  Same
 * layout, flags and diag_shift as qmlg_gaussian_kernel.  Synchronises the stream
 * once (the bound needs max |x| on the host).  ws: the size call below.
 */
size_t qmlg_gaussian_kernel_emulated_workspace_size(int na, int nb, int d, int flags);
int qmlg_gaussian_kernel_emulated(const double *A, int64_t lda, int na, const double *B,
                                  int64_t ldb, int nb, int d, double sigma, double *K,
                                  int64_t ldk, int flags, double diag_shift, void *workspace,
                                  size_t ws_bytes, void *stream);

/*
 * The Sargan kernel (qml/fkernels.f90:487-531) from exact fixed-point L1 sums: the
 * qmlg_laplacian_kernel_fixed grid and kernel with the Sargan polynomial in the
 * epilogue.  For gammas >= 0 the grid's bound on t = d / sigma is tightened by
 * 1 + ng max(1, sum gamma), which keeps every entry within 0.5e-12 relative; a
 * negative or non-finite gamma, input that is not finite and a bound the grid
 * cannot meet take qmlg_sargan_kernel.  gammas: device array (read back once).
 * Arguments as qmlg_sargan_kernel.  ws: qmlg_sargan_kernel_fixed_workspace_size.
 */
size_t qmlg_sargan_kernel_fixed_workspace_size(int na, int nb, int d, int flags);
int qmlg_sargan_kernel_fixed(const double *A, int64_t lda, int na, const double *B, int64_t ldb,
                             int nb, int d, double sigma, const double *gammas, int ng, double *K,
                             int64_t ldk, int flags, double diag_shift, void *workspace,
                             size_t ws_bytes, void *stream);

/*
 * The Matern L2 kernel (qml/fkernels.f90:426-484) of order 1 or 2 on the tensor
 * cores: the Gaussian tile kernel's d^2 = |a|^2 + |b|^2 - 2 a.b with the Matern
 * epilogue.  Both orders are flat at d = 0, so |K - K_exact| / K stays below
 * 0.25e-12 whenever the digit bound allows (the same test as the Gaussian's, with
 * three times the margin); otherwise, for order 0 and for input that is not
 * finite, qmlg_matern_kernel_l2 runs.  Arguments as qmlg_matern_kernel_l2.
 * ws: qmlg_matern_kernel_l2_emulated_workspace_size(na, nb, d, flags).
 */
size_t qmlg_matern_kernel_l2_emulated_workspace_size(int na, int nb, int d, int flags);
int qmlg_matern_kernel_l2_emulated(const double *A, int64_t lda, int na, const double *B,
                                   int64_t ldb, int nb, int d, double sigma, int order, double *K,
                                   int64_t ldk, int flags, double diag_shift, void *workspace,
                                   size_t ws_bytes, void *stream);

/*
 * The linear kernel K = A B^T (qml/fkernels.f90:403-423) on the tensor cores: the
 * Gaussian tile kernel with the dot product itself as the entry.  Every row is cut
 * into eight 7-bit digit planes; the plane products are summed exactly in integers
 * and scaled to K with one rounding.  |K - A B^T| <= 2^(eA + eB - 56) * kp * 9/4 for
 * each entry, with 2^eA > max|a_j| and 2^eB > max|b_i| over the two rows and kp = d
 * rounded up to 64.  Layouts, flags and diag_shift as qmlg_linear_kernel; input
 * that is not finite takes qmlg_linear_kernel.
 * ws: qmlg_linear_kernel_emulated_workspace_size(na, nb, d, flags).
 */
size_t qmlg_linear_kernel_emulated_workspace_size(int na, int nb, int d, int flags);
int qmlg_linear_kernel_emulated(const double *A, int64_t lda, int na, const double *B,
                                int64_t ldb, int nb, int d, double *K, int64_t ldk, int flags,
                                double diag_shift, void *workspace, size_t ws_bytes, void *stream);

/*
 * Laplacian kernel with the L1 distances summed exactly in 64-bit fixed point on
 * the integer pipes: features rounded once to multiples of 2^-F (F from max |x|
 * and d so that sums cannot overflow), |a - b| summed exactly, converted to FP64
 * once.  Entries stay within 1e-12 relative of the FP64 kernel (bound
 * d * 2^-F / sigma <= 0.5e-12, else the FP64 kernel runs); K is exactly
 * symmetric.  Same layout and flags as qmlg_laplacian_kernel.  Synchronises the
 * stream once (max |x|).
 */
size_t qmlg_laplacian_kernel_fixed_workspace_size(int na, int nb, int d, int flags);
int qmlg_laplacian_kernel_fixed(const double *A, int64_t lda, int na, const double *B,
                                int64_t ldb, int nb, int d, double sigma, double *K, int64_t ldk,
                                int flags, double diag_shift, void *workspace, size_t ws_bytes,
                                void *stream);

/*
 * Capture-safe qmlg_laplacian_kernel_fixed (replaces flaplacian_kernel,
 * qml/fkernels.f90:374-400, in batched and graph-recorded fits): no host
 * synchronisation and no host decision.  The fixed-point grid and its 1e-12 bound
 * are decided on the device; when the bound fails, the FP64 kernel (launched beside
 * the fixed-point one, and returning at once otherwise) writes K and 8 is ORed into
 * the caller's device int *d_flag (may be NULL).  K is always written.  Same layout,
 * flags and workspace size as qmlg_laplacian_kernel_fixed.
 */
int qmlg_laplacian_kernel_fixed_async(const double *A, int64_t lda, int na, const double *B,
                                      int64_t ldb, int nb, int d, double sigma, double *K,
                                      int64_t ldk, int flags, double diag_shift, int *d_flag,
                                      void *workspace, size_t ws_bytes, void *stream);

/*
 * Capture-safe qmlg_gaussian_kernel_emulated: no host synchronisation (so it can
 * be recorded into a CUDA graph); always 8 digit planes; the 1e-12 bound is
 * checked on the device and a failure ORs 8 into the caller's device int
 * *d_flag (then recompute with qmlg_gaussian_kernel); 1/2/4 = a bounded
 * tensor-core wait gave up.  Workspace as qmlg_gaussian_kernel_emulated.
 */
int qmlg_gaussian_kernel_emulated_async(const double *A, int64_t lda, int na, const double *B,
                                        int64_t ldb, int nb, int d, double sigma, double *K,
                                        int64_t ldk, int flags, double diag_shift, int *d_flag,
                                        void *workspace, size_t ws_bytes, void *stream);

/* ---- prediction ----------------------------------------------------------- */

#define QMLG_KIND_GAUSSIAN 0
#define QMLG_KIND_LAPLACIAN 1

/*
 * yhat[i] = sum_j Ks[j + i*ldk] * alpha[j] for a materialised prediction kernel
 * Ks(ntrain, ntest): the np.dot(Ks.T, alpha) of tests/test_energy_krr_cmat.py:109.
 */
int qmlg_predict_gemv(const double *Ks, int64_t ldk, int ntrain, int ntest,
                      const double *alpha, double *yhat, void *stream);

/*
 * Fused prediction: yhat[i] = sum_j k(Xtrain_j, Xtest_i) * alpha[j] without
 * materialising Ks.  Partial sums per training tile go to the workspace and are
 * reduced in a fixed order, so the result is deterministic.
 */
size_t qmlg_predict_workspace_size(int ntrain, int ntest);
int qmlg_predict_fused(int kind, const double *Xtrain, int64_t ldtrain, int ntrain,
                       const double *Xtest, int64_t ldtest, int ntest, int d, double sigma,
                       const double *alpha, double *yhat, void *workspace, size_t ws_bytes,
                       void *stream);

/*
 * Laplacian prediction yhat = K(Xtest, Xtrain) alpha with the L1 sums in 64-bit
 * fixed point, as qmlg_laplacian_kernel_fixed (same grid, same bound: every kernel
 * entry within 1e-12 of FP64), fused like qmlg_predict_fused: no kernel matrix is
 * written and the partial sums are reduced in a fixed order.  When the data do not
 * fit the fixed-point grid it runs qmlg_predict_fused's FP64 kernel.  The call
 * reads two maxima back to the host (it synchronises the stream once).
 * ws: qmlg_predict_laplacian_fixed_workspace_size(ntrain, ntest, d).
 */
size_t qmlg_predict_laplacian_fixed_workspace_size(int ntrain, int ntest, int d);
int qmlg_predict_laplacian_fixed(const double *Xtrain, int64_t ldtrain, int ntrain,
                                 const double *Xtest, int64_t ldtest, int ntest, int d,
                                 double sigma, const double *alpha, double *yhat,
                                 void *workspace, size_t ws_bytes, void *stream);

/*
 * qmlg_predict_laplacian_fixed without any host synchronisation, for serving loops
 * (the np.dot(Ks.T, alpha) of tests/test_energy_krr_cmat.py:109 with the Laplacian
 * Ks of qml/kernels.py:36-63): the grid is decided on the device; when its bound
 * fails the FP64 fused kernel (launched beside the fixed-point one) writes yhat and
 * 8 is ORed into *d_flag (may be NULL).  yhat is always written.  Same workspace
 * size as qmlg_predict_laplacian_fixed.
 */
int qmlg_predict_laplacian_fixed_async(const double *Xtrain, int64_t ldtrain, int ntrain,
                                       const double *Xtest, int64_t ldtest, int ntest, int d,
                                       double sigma, const double *alpha, double *yhat,
                                       int *d_flag, void *workspace, size_t ws_bytes,
                                       void *stream);

/*
 * qmlg_predict_fused without a workspace, for callers that cannot allocate device
 * memory (for example a serving process whose memory manager reserves all of its
 * HBM at start-up and forbids later cudaMalloc calls, which synchronise the device
 * and can fail under fragmentation).  No counterpart in the reference: the
 * reference has no device memory at all.
 * Scratch lives in a fixed 32 MiB array inside the library (reserved on every GPU
 * that loads it, until exit); the call needs ceil(ntrain/64) * ntest <= 4194304
 * and returns QMLG_E_TOO_LARGE beyond that.  It allocates nothing.  The first call
 * on a device looks up the array's device address (cudaGetSymbolAddress) with that
 * device current, so make that first call before any stream capture; the stream
 * must belong to the current device.  All calls share the array: calls whose work
 * overlaps on the GPU race and must be serialised by the caller.
 */
int qmlg_predict_fused_noalloc(int kind, const double *Xtrain, int64_t ldtrain, int ntrain,
                               const double *Xtest, int64_t ldtest, int ntest, int d,
                               double sigma, const double *alpha, double *yhat, void *stream);

/*
 * Gaussian prediction yhat[i] = sum_j k(Xtrain_j, Xtest_i) alpha[j] with the kernel
 * formed on the tensor cores as in qmlg_gaussian_kernel_emulated and reduced in
 * the epilogue (Ks is never written); deterministic fixed-order reduction.
 */
size_t qmlg_predict_emulated_workspace_size(int ntrain, int ntest, int d);
int qmlg_predict_emulated(const double *Xtrain, int64_t ldtrain, int ntrain,
                          const double *Xtest, int64_t ldtest, int ntest, int d, double sigma,
                          const double *alpha, double *yhat, void *workspace, size_t ws_bytes,
                          void *stream);

/*
 * qmlg_predict_emulated without any host synchronisation, for serving loops that
 * keep several streams busy: always 8 digit planes; the accuracy bound and any
 * bounded-wait timeout are checked on the device and reported by OR-ing into the
 * caller's device int *d_flag (8 = the 1e-12 bound is not met for this sigma and
 * data, so recompute with qmlg_predict_fused; 1/2/4 = a tensor-core wait gave
 * up).  Clear *d_flag before the call; read it after the stream has completed.
 * Same workspace size as qmlg_predict_emulated.
 */
int qmlg_predict_emulated_async(const double *Xtrain, int64_t ldtrain, int ntrain,
                                const double *Xtest, int64_t ldtest, int ntest, int d,
                                double sigma, const double *alpha, double *yhat, int *d_flag,
                                void *workspace, size_t ws_bytes, void *stream);

/* ---- Cholesky solve ------------------------------------------------------- */

#define QMLG_PREC_FP64 0   /* plain FP64 blocked Cholesky (LAPACK dpotrf semantics) */
#define QMLG_PREC_MIXED 1  /* emulated-FP64 tensor-core factor + exact-residual refinement */

typedef struct QmlgSolveReport {
    int precision_used;     /* QMLG_PREC_* of the factor the answer came from */
    int info;               /* Cholesky info of that factor (0 = ok) */
    int outer_iterations;   /* refinement steps taken */
    int inner_iterations;   /* total GMRES iterations */
    int fell_back;          /* 1 if the mixed path gave up and refactorised in FP64 */
    double shift;           /* diagonal shift used for the low-precision factor */
    double backward_error;  /* |r|_2 / (|A|_F |x|_2 + |y|_2) of the returned x */
    double last_correction; /* |dx|_2 / |x|_2 of the last refinement step */
} QmlgSolveReport;

typedef struct QmlgRefineOpts {
    int max_outer;          /* refinement steps (default 10) */
    int max_inner;          /* not used: each step solves with the factor directly */
    double tol;             /* stop when |dx|/|x| <= tol (default 1e-15) */
    double shift;           /* not used: the factor takes no extra diagonal shift */
    int allow_fallback;     /* refactorise in FP64 when refinement stalls (default 1) */
    int slices;             /* digit planes of the mixed factor's tensor-core products,
                               4..8 (0 = 8).  Fewer planes give a faster factor with a
                               larger error; when refinement cannot recover from it (an
                               ill-conditioned matrix) the solve stalls and takes the
                               FP64 refactorisation (report->fell_back = 1). */
} QmlgRefineOpts;

/*
 * Cholesky factor in place, LAPACK dpotrf("U") semantics on a column-major
 * n x n matrix A (leading dimension lda): the upper triangle is overwritten with
 * U (A = U^T U), the strictly lower triangle is left untouched.  lambda is added
 * to the diagonal before factorising (0 for the reference).  Returns info > 0
 * on a non-positive leading minor.  Replaces the dpotrf call of fcho_solve
 * (qml/fcho_solve.f90:35).  ws: qmlg_cholesky_workspace_size(n).
 */
size_t qmlg_cholesky_workspace_size(int n);
int qmlg_cholesky(double *A, int n, int64_t lda, double lambda, void *workspace,
                  size_t ws_bytes, void *stream);

/*
 * The same factorisation with the O(n^3) trailing updates emulated to FP64 accuracy
 * on the bf16 tensor cores (tcgen05): every panel row is scaled by a power of two
 * and cut into 8 base-128 digits; the digit-plane products are summed exactly in
 * FP32 tensor memory and merged into FP64 once per element.  Diagonal blocks and
 * panel solves stay in FP64.  Same storage, same info as qmlg_cholesky; the factor
 * agrees with it to FP64 rounding level (not bit for bit).  Returns
 * QMLG_E_TIMEOUT if a bounded device-side wait gave up.
 */
size_t qmlg_cholesky_mixed_workspace_size(int n);
int qmlg_cholesky_mixed(double *A, int n, int64_t lda, double lambda, void *workspace,
                        size_t ws_bytes, void *stream);

/*
 * The trailing update of qmlg_cholesky_mixed on its own: C <- C - P P^T on the
 * lower triangle of the row-major n x n matrix C (the column-major upper one),
 * P row-major n x k (k <= 512), the products emulated to FP64 accuracy with 8
 * digit planes on the tensor cores.  Exposed for timing and for callers that
 * assemble their own blocked factorisations.
 */
size_t qmlg_syrk_emulated_workspace_size(int n, int k);
int qmlg_syrk_emulated(double *C, int64_t ldc, int n, const double *P, int64_t ldp, int k,
                       void *workspace, size_t ws_bytes, void *stream);

/*
 * x = (U^T U)^{-1} y with U from qmlg_cholesky: dpotrs("U", nrhs=1)
 * (qml/fcho_solve.f90:46).  x and y may alias.
 */
int qmlg_cholesky_solve_factored(const double *U, int n, int64_t lda, const double *y,
                                 double *x, void *stream);

/*
 * Full solve (A + lambda I) x = y, the fcho_solve of qml/fcho_solve.f90:23-52 with
 * the KRR lambda folded in.  precision QMLG_PREC_FP64 factorises A in place like
 * the reference (upper triangle overwritten); QMLG_PREC_MIXED factorises in place
 * the same way with qmlg_cholesky_mixed, then refines with an exact
 * residual read from the untouched triangle, and falls back to a plain FP64
 * refactorisation when refinement stalls (opts->allow_fallback).  In both modes
 * the column-major strictly lower triangle of A is never written.  opts and
 * report may be NULL.
 * The call synchronises the stream (refinement decisions are taken on the host).
 */
size_t qmlg_solve_workspace_size(int n, int precision);
int qmlg_solve(double *A, int n, int64_t lda, const double *y, double *x, double lambda,
               int precision, const QmlgRefineOpts *opts, QmlgSolveReport *report,
               void *workspace, size_t ws_bytes, void *stream);

/*
 * Capture-safe mixed solve (A + lambda I) x = y for batched, graph-recorded
 * work: the qmlg_cholesky_mixed factorisation, one solve and exactly
 * refine_steps exact-residual refinement steps, with no host synchronisation and
 * no host decision.  Results stay on the device: d_status[0] = Cholesky info
 * (0 = ok), d_status[1] = bounded-wait flags (bit 1: a tensor-core pipeline
 * wait, bit 2: a triangular-solve wait gave up); d_correction (optional, 2
 * doubles) = |dx|^2 and |x|^2 of the last step.  The column-major upper
 * triangle of A receives the factor as in qmlg_cholesky.
 */
size_t qmlg_solve_async_workspace_size(int n);
int qmlg_solve_async(double *A, int n, int64_t lda, const double *y, double *x, double lambda,
                     int refine_steps, int *d_status, double *d_correction, void *workspace,
                     size_t ws_bytes, void *stream);

/*
 * Batched KRR fits: many independent fits of uneven size, as the learning curves and
 * sigma x lambda grids of docs/source/tutorial.rst:168-174 run them, each the
 * gaussian_kernel / laplacian_kernel + K[diag] += lambda + cho_solve sequence of
 * tests/test_energy_krr_cmat.py:97-106 (qml/kernels.py:36-92, qml/fcho_solve.f90:23-52).
 * Every phase is one grouped launch over all fits instead of one launch per fit:
 *   - the symmetric Gaussian kernel matrices of every Gaussian fit, on the tensor
 *     cores as qmlg_gaussian_kernel_emulated_async (8 digit planes; a fit whose data
 *     miss the 1e-12 bound gets 8 in its flags); Laplacian fits take
 *     qmlg_laplacian_kernel_fixed_async each;
 *   - the mixed factorisation in lockstep 64-column steps: FP64 diagonal blocks of
 *     every fit in one launch, their panel solves in one, the K = 64 updates in one
 *     tensor-core launch, and every 512 columns one tensor-core launch for all
 *     trailing matrices;
 *   - the block inverses, then the triangular solves one 64-row block per launch for
 *     all fits at once, and refine_steps exact-residual refinement steps.
 * No host synchronisation and no host decision: the call can be recorded into a CUDA
 * graph.  All pointers are device pointers except the problem array itself, which
 * is read during the call only.  At most 128 fits per call.
 *   K       n x n column-major buffer per fit: receives K in its strictly lower
 *           triangle (the factor in the upper one, as qmlg_cholesky)
 *   status  device int[2] per fit: [0] Cholesky info (0 = ok); [1] flags: 8 = the
 *           kernel's fast path missed its bound (Gaussian: refit that fit with
 *           qmlg_solve; Laplacian: the FP64 kernel formed K, nothing to do),
 *           1/2/4 = a bounded tensor-core wait gave up
 *   correction  optional device double[2]: |dx|^2 and |x|^2 of the last step
 * tile_cols: i-columns per tensor-core tile of the factorisation's updates, 64 or
 * 32; trsm_rows: rows per CTA of the panel solves, 32..128 (multiple of 8).  0 takes
 * the defaults (64, 128); a batch autotuner picks them per size bucket.
 */
typedef struct QmlgBatchProblem {
    const double *X;      /* n x d representations, row-major */
    int64_t ldx;
    int n;
    int kind;             /* QMLG_KIND_GAUSSIAN or QMLG_KIND_LAPLACIAN */
    double sigma;
    double lambda;
    const double *y;      /* n labels */
    double *alpha;        /* n weights, written */
    double *K;            /* n x n, leading dimension n */
    int *status;          /* device int[2] */
    double *correction;   /* device double[2] or NULL */
} QmlgBatchProblem;

size_t qmlg_fit_batched_workspace_size(const QmlgBatchProblem *problems, int count, int d);
int qmlg_fit_batched_async(const QmlgBatchProblem *problems, int count, int d, int refine_steps,
                           int tile_cols, int trsm_rows, void *workspace, size_t ws_bytes,
                           void *stream);

/*
 * Inverse of a symmetric positive-definite matrix: Ainv (column-major, ldi) =
 * A^-1, both triangles written.  Reads A's column-major lower triangle, as
 * dpotrf("L") + dpotri("L") in fcho_invert (qml/fcho_solve.f90:54-73), bound by
 * qml.math.cho_invert (qml/math.py:33-58).  Computed as the Schur complement left
 * by the first ceil64(n) Cholesky pivots of [[A, I], [I, 0]] (A padded with an
 * identity), with the FP64 (QMLG_PREC_FP64) or the tensor-core (QMLG_PREC_MIXED)
 * factorisation.  Returns 0, or LAPACK's info (> 0: the leading minor of that order
 * is not positive definite; Ainv is then unusable, where the reference prints a
 * warning and returns whatever dpotri produced).  A is not modified.
 */
size_t qmlg_cho_invert_workspace_size(int n, int precision);
int qmlg_cho_invert(const double *A, int n, int64_t lda, double *Ainv, int64_t ldi, int precision,
                    void *workspace, size_t ws_bytes, void *stream);

/*
 * Symmetric (possibly indefinite) solve A x = y by Bunch-Kaufman diagonal pivoting,
 * restating dsytrf("L") + dsytrs("L") as fbkf_solve calls them
 * (qml/fcho_solve.f90:115-150), bound by qml.math.bkf_solve (qml/math.py:125-164).
 * Reads A's column-major lower triangle; A is not modified.  Returns 0, or LAPACK's
 * info (> 0: D(info, info) is exactly zero, x is then unusable, where the reference
 * prints a warning).  Above n = 256 (outside stream capture) the factorisation is
 * dsytrf's blocked form (dlasyf panels) with the trailing updates as emulated-FP64
 * tensor-core products, and x is refined once on the FP64 residual y - A x; the
 * call waits on the stream once per 64-column panel.
 */
size_t qmlg_bkf_solve_workspace_size(int n);
int qmlg_bkf_solve(const double *A, int n, int64_t lda, const double *y, double *x,
                   void *workspace, size_t ws_bytes, void *stream);

/*
 * Inverse of a symmetric (possibly indefinite) matrix by Bunch-Kaufman pivoting, as
 * dsytrf("L") + dsytri("L") in fbkf_invert (qml/fcho_solve.f90:76-112), bound by
 * qml.math.bkf_invert (qml/math.py:100-122): Ainv (column-major, ldi, both
 * triangles) = A^-1, computed as the Schur complement left by n pivot steps on
 * [[A, I], [I, 0]] with the pivots searched among A's rows.  Returns 0 or info.
 * Above n = 128 (outside stream capture) the factorisation is blocked as in
 * qmlg_bkf_solve, with FP64 trailing updates.
 */
size_t qmlg_bkf_invert_workspace_size(int n);
int qmlg_bkf_invert(const double *A, int n, int64_t lda, double *Ainv, int64_t ldi,
                    void *workspace, size_t ws_bytes, void *stream);

/*
 * r = y - (A + lambda I) x summed exactly (every product formed from the 53-bit
 * significands and added into 256-bit fixed point on the integer pipes) and
 * rounded once: each r[i] is the correctly rounded exact residual, independent of
 * the summation order.  Uses A's strictly lower triangle (column-major, untouched
 * by the factorisation) and the diagonal vector diag (the diagonal of A before
 * factorising).  The name is kept from its first, double-double form.
 * ws: qmlg_residual_workspace_size(n).
 */
size_t qmlg_residual_workspace_size(int n);
int qmlg_residual_dd(const double *A, int n, int64_t lda, const double *diag, double lambda,
                     const double *x, const double *y, double *r, void *workspace,
                     size_t ws_bytes, void *stream);

/*
 * Self-test of the bounded device-side waits (no reference counterpart): one CTA
 * polls entries of a triangular-solve output that nothing ever writes, with the
 * same wait routine the cooperative solves use.  The wait gives up after its poll
 * limit (about a second) and the call returns QMLG_E_TIMEOUT; the context stays
 * usable.  ws: qmlg_selftest_wait_timeout_workspace_size().
 */
size_t qmlg_selftest_wait_timeout_workspace_size(void);
int qmlg_selftest_wait_timeout(void *workspace, size_t ws_bytes, void *stream);

/*
 * The exp of the tensor-core Gaussian epilogues, element-wise (no reference
 * counterpart; exposed so that its accuracy can be checked against the library exp):
 * y[i] = exp(x[i]) for x[i] <= 0, fixed-point table reduction, at most a few ulp;
 * x[i] > 0 reads as 0 (the epilogue clamps distances that round below 0).
 */
int qmlg_epilogue_exp(const double *x, double *y, int n, void *stream);

/* ---- files ------------------------------------------------------------ */

/*
 * Reads many files on host threads (the open/readlines of each
 * qml/compound.py:296-326 Compound.read_xyz call).  HOST pointers; no stream.
 * paths: nfiles NUL-terminated names.  With buf == NULL it sets sizes[f] to the
 * size of file f (-1 when it is not a regular file that stat can see).  The caller
 * then places the files (starts, nfiles+1) and calls again with buf: file f is read
 * into buf[starts[f] .. starts[f+1]), and status[f] = 1 when it could not be read
 * in full or its size no longer matches sizes[f] (0 otherwise).  nthreads <= 0:
 * one per hardware thread.  Returns 0 or QMLG_E_ARG.
 */
int qmlg_read_files(const char *const *paths, int nfiles, int nthreads, int64_t *sizes,
                    char *buf, const int64_t *starts, int *status);

/*
 * Parses many XYZ files on host threads (replaces the per-file
 * qml/compound.py:296-326 Compound.read_xyz loop a caller runs over a dataset).
 * HOST pointers; no stream.  File f is text[starts[f] .. starts[f+1]); each is read
 * as read_xyz reads it: the atom count on line 1, a comment line, then one atom per
 * line (symbol x y z) until the count, the end of the file or a line with fewer than
 * four fields.  Outputs: offsets (nfiles+1) = the files' atom ranges in
 * charges (capacity) and coordinates (capacity x 3, row-major); status[f] = 0 when
 * file f was parsed, 1 when this parser does not accept it (non-ASCII bytes, an
 * atom count that is not a plain decimal integer >= 0, an element outside the
 * qml/data.py:23 table, a number strtod does not read in full).  The caller parses
 * a flagged file the reference's way, which gives its result or its error.  At
 * most (line breaks in text + nfiles) atoms exist, so that capacity always suffices.
 * nthreads <= 0: one per hardware thread.  Returns 0, QMLG_E_ARG, or
 * QMLG_E_TOO_LARGE when the atoms exceed capacity.
 */
int qmlg_parse_xyz(const char *text, const int64_t *starts, int nfiles, int nthreads,
                   int64_t *offsets, int *status, double *charges, double *coordinates,
                   int64_t capacity);

#ifdef __cplusplus
}
#endif

#endif /* QMLG_H */
