/*
 * rest_tensors_gb300.h - C ABI of the GB300 (sm_103a) dense RI contraction path.
 *
 * Two families of entry points:
 *
 *  1. Drop-in replacements for the reference's Fortran seam, with the exact
 *     Fortran calling convention (every argument by reference, trailing
 *     underscore, host pointers, column-major storage).  A build that links
 *     this library instead of librestmatr.so serves the unchanged Rust
 *     callers (RIFull::ao2mo, _dgemm).
 *
 *  2. rt_* functions on device pointers.  They take a cudaStream_t (passed as
 *     void*), return rt_status, never abort and never trap.  Arrays are
 *     float64, column-major, in the reference's layouts:
 *       ri3ao  RIFull [nb, nb, naux]          B[mu + nb*nu + nb*nb*P]       (src/ri.rs:19-40)
 *       C      MatrixFull [nb, ns]            C[mu + nb*p]                  (src/matrix/mod.rs:473-480)
 *       ri3mo  RIFull [naux, ns, ns]          R[P + naux*p + naux*ns*q]     (src/ri.rs:382-408)
 *       ov     [nocc, nvir, naux]             O[i + nocc*a + nocc*nvir*P]
 *       D,J,K  MatrixFull [nb, nb]
 *
 * Precision forms (rt_form):
 *   RT_FORM_FP64   IEEE float64 throughout (CUDA-core DFMA).
 *   RT_FORM_SPLIT  each float64 operand split into `nslices` signed 7-bit
 *                  digits held exactly in BF16, multiplied on the tcgen05
 *                  tensor cores with exact FP32 accumulation, recombined
 *                  exactly in 64-bit integers and rounded once to float64.
 *                  Inputs must be finite; values below 2^-1022 are flushed.
 *
 * Calls on one device may come from several host threads; each call is
 * stream-ordered on the stream it is given.
 */
#ifndef REST_TENSORS_GB300_H
#define REST_TENSORS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int rt_status;
#define RT_OK 0
#define RT_ERR_INVALID_ARG 1
#define RT_ERR_CUDA 2
#define RT_ERR_NO_MEMORY 3
#define RT_ERR_UNSUPPORTED 4
#define RT_ERR_NONFINITE 5
#define RT_ERR_TIMEOUT 6
#define RT_ERR_NOT_CONVERGED 7

#define RT_FORM_FP64 0
#define RT_FORM_SPLIT 1

/* Library version, (major << 16) | minor. */
int rt_version(void);
/* Text for a status code. */
const char* rt_status_string(rt_status s);
/* Status and message of the most recent failing call on this host thread. */
rt_status rt_last_status(void);
const char* rt_last_error(void);
/* Synchronise `stream` and report device-side findings of kernels launched
 * since the last check (RT_ERR_NONFINITE for a non-finite input to the split
 * form, RT_ERR_TIMEOUT for an exhausted bounded wait); clears them. */
rt_status rt_sync_status(void* stream);

/* ------------------------------------------------------------------------
 * Drop-in Fortran seam (host pointers).
 *
 * Precision form of the three drop-ins: read once per process from the
 * environment, RT_FORM = fp64 (default) or split, and RT_NSLICES = 3..8
 * (digits per float64 in the split form, default 7).  Unchanged callers get the
 * float64 form; a deployment opts in to the split form without relinking.
 * An unrecognised value makes every drop-in call fail (rt_last_status() is
 * RT_ERR_INVALID_ARG) instead of running another form.  No counterpart in the
 * reference, whose seam is float64 only.
 * ------------------------------------------------------------------------ */

/* Replaces ri_ao2mo_f_ (src/external_libs/ffi_restmatr.rs:5-11, implemented at
 * src/external_libs/restmatr.f90:158-194):
 *   ri3mo[P,p,q] = sum_{mu,nu} eigenvector[mu,p] ri3fn[mu,nu,P] eigenvector[nu,q]
 * ri3mo is [num_auxbas, num_states, num_states] (P fastest).  Runs
 * rt_ri_ao2mo_host in the seam's form on the per-thread default stream.
 * Failures are reported through rt_last_status()/rt_last_error() (the Fortran
 * subroutine has no return value) and ri3mo is then left zero-filled. */
void ri_ao2mo_f_(const double* eigenvector, const double* ri3fn, double* ri3mo, const int* num_states,
                 const int* num_basis, const int* num_auxbas);

/* Replaces general_dgemm_f_ (src/external_libs/ffi_restmatr.rs:13-24,
 * restmatr.f90:63-107): on column-major host matrices,
 *   C[rc, cc] = alpha * op_a(A[ra, ca]) * op_b(B[rb, cb]) + beta * C[rc, cc]
 * with blocks given by 0-based start and length.  In the split form the
 * product is formed from digit planes and alpha, beta are applied in float64
 * (beta = 0 does not read C). */
void general_dgemm_f_(const double* matr_a, const int* rows_a, const int* columns_a, const int* start_row_a,
                      const int* len_row_a, const int* start_column_a, const int* len_column_a, const char* opa,
                      const double* matr_b, const int* rows_b, const int* columns_b, const int* start_row_b,
                      const int* len_row_b, const int* start_column_b, const int* len_column_b, const char* opb,
                      double* matr_c, const int* rows_c, const int* columns_c, const int* start_row_c,
                      const int* len_row_c, const int* start_column_c, const int* len_column_c,
                      const double* alpha, const double* beta);

/* Replaces special_dgemm_f_01_ (src/external_libs/ffi_restmatr.rs:25-33,
 * restmatr.f90:111-154; Rust wrapper src/external_libs/mod.rs:85-99), the
 * O_V * V^{-1/2} step of the ri3fn preparation.  For every y-slice of the
 * column-major host tensor ten3_a[x_a, y_a, z_a]:
 *   T = ten3_a[sx:sx+lx, y, sz:sz+lz]
 *   T <- alpha * T * matr_b[rb:rb+lz, cb:cb+lz] + beta * T
 * with 0-based starts and lengths.  The block of matr_b must be lz x lz.
 * i_y_a is accepted and ignored, as in the Fortran, which loops over all
 * y-slices.  The Fortran body hands one buffer to dgemm as both A and C; this
 * entry computes the product those arguments describe, from an unaliased
 * copy.  Runs in the seam's form.  Failures are reported through
 * rt_last_status() / rt_last_error() and leave ten3_a unchanged. */
void special_dgemm_f_01_(double* ten3_a, const int* x_a, const int* y_a, const int* z_a, const int* start_x_a,
                         const int* len_x_a, const int* i_y_a, const int* start_z_a, const int* len_z_a,
                         const double* matr_b, const int* rows_b, const int* columns_b, const int* start_row_b,
                         const int* len_row_b, const int* start_column_b, const int* len_column_b,
                         const double* alpha, const double* beta);

/* ------------------------------------------------------------------------
 * Device-pointer API.
 * ------------------------------------------------------------------------ */

/* General column-major float64 GEMM on the device, lapack_dgemm semantics
 * (src/matrix/matrix_blas_lapack.rs:739-774):
 *   C = alpha * op(A) * op(B) + beta * C,  op in {'N','T'}. */
rt_status rt_dgemm(char opa, char opb, int m, int n, int k, double alpha, const double* A, int lda, const double* B,
                   int ldb, double beta, double* C, int ldc, void* stream);

/* The same product in the split-precision form: C = op(A) * op(B) (alpha = 1,
 * beta = 0), each float64 operand cut into `nslices` BF16 digit planes per row
 * of op(A) and column of op(B), multiplied on the tcgen05 tensor cores and
 * recombined exactly.  Inputs must be finite.  A call with B == A, ldb == lda,
 * m == n and opposite ops (A A^T or A^T A) is computed as a symmetric rank-k
 * update: one set of digit planes, one triangle, mirrored. */
rt_status rt_dgemm_split(char opa, char opb, int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                         double* C, int ldc, int nslices, void* stream);

/* special_dgemm_f_01_ on device memory and a stream: the same operation on
 * ten3_a[x_a, y_a, z_a] and matr_b[rows_b, columns_b], in place.  form
 * RT_FORM_FP64, or RT_FORM_SPLIT (nslices 3..8), whose product runs on the
 * tensor cores and then applies alpha and beta in float64; its inputs must be
 * finite (rt_sync_status then reports RT_ERR_NONFINITE otherwise).  Scratch:
 * at most 8 GB of staged y-slices (plus the split form's digit planes). */
rt_status rt_special_dgemm_01(double* ten3_a, int x_a, int y_a, int z_a, int start_x_a, int len_x_a, int start_z_a,
                              int len_z_a, const double* matr_b, int rows_b, int columns_b, int start_row_b,
                              int len_row_b, int start_column_b, int len_column_b, double alpha, double beta,
                              int form, int nslices, void* stream);

/* Full AO->MO transform, RIFull::ao2mo (src/ri.rs:356-408):
 *   ri3mo[P,p,q] = (C^T B^P C)[p,q],  C = [nb, ns], B = [nb, nb, naux] symmetric in (mu, nu).
 * form RT_FORM_FP64 or RT_FORM_SPLIT (nslices 3..8; ignored for FP64). */
rt_status rt_ri_ao2mo(const double* C, const double* B, double* ri3mo, int nb, int ns, int naux, int form,
                      int nslices, void* stream);

/* Occupied-virtual transform plus RI-K from one shared half-transform
 * X^P = B^P C_occ (the first dgemm of restmatr.f90:183-185):
 *   ov[i,a,P] = (C_occ^T B^P C_vir)[i,a]      (i fastest; C_vir = C + nb*nocc)
 *   K[mu,nu]  = sum_P (X^P X^P^T)[mu,nu]
 * C = [nb, nocc + nvir].  Either output pointer may be NULL to skip it. */
rt_status rt_ri_ov_k(const double* C, const double* B, int nb, int naux, int nocc, int nvir, double* ov, double* K,
                     int form, int nslices, void* stream);

/* Allocation-free float64 form of rt_ri_ov_k, for callers that cannot
 * allocate device memory while they run: a host runtime that has handed the
 * GPU's memory to a fixed arena it manages itself, or a serving path on which
 * cudaMalloc/cudaFree, and the device synchronisation they imply, are not
 * allowed.  It has no counterpart in the reference.  The half-
 * transform goes through one fixed 32 MiB device array that the library
 * holds on every GPU that loads it, so nb*nocc may be at most 4,194,304
 * (larger requests fail with RT_ERR_INVALID_ARG); the aux slabs stream through
 * it in blocks.  The first call on each device looks up the array's address
 * (cudaGetSymbolAddress).  All calls share the array: calls whose kernels
 * overlap on the GPU race. */
rt_status rt_ri_ov_k_fp64_noalloc(const double* C, const double* B, int nb, int naux, int nocc, int nvir, double* ov,
                                  double* K, void* stream);

/* ri3ao prepared for repeated split-form ov + RI-K: its BF16 digit planes and
 * row exponents as the A operand of the half-transform X^P = B^P C_occ, made
 * once and reused by every rt_ri_ov_k_prepared call with new orbitals.  In
 * REST's SCF loop ri3fn is fixed while C changes, so each iteration then skips
 * slicing the three-centre tensor (it still reads its digit planes).  No
 * counterpart in the reference; the results are bitwise those of rt_ri_ov_k
 * in the split form with the same nslices.  The planes take about
 * 2 nslices nb^2 naux bytes on the device that made them
 * (rt_ri3ao_prepared_bytes), held until rt_ri3ao_release.  rt_ri3ao_prepare
 * synchronises `stream`, so the handle is ready on return; B is not referenced
 * afterwards. */
typedef struct rt_ri3ao_prepared rt_ri3ao_prepared;
rt_status rt_ri3ao_prepare(const double* B, int nb, int naux, int nslices, rt_ri3ao_prepared** out, void* stream);
rt_status rt_ri3ao_prepared_bytes(const rt_ri3ao_prepared* h, long long* bytes);
rt_status rt_ri_ov_k_prepared(const rt_ri3ao_prepared* h, const double* C, int nocc, int nvir, double* ov, double* K,
                              void* stream);
rt_status rt_ri3ao_release(rt_ri3ao_prepared* h);

/* One molecule of a batch: device pointers and sizes as for rt_ri_ov_k. */
typedef struct {
    const double* C;
    const double* B;
    double* ov;
    double* K;
    int nb, naux, nocc, nvir;
} rt_ri_problem;

/* Launch options of the split form.  fuse: form the ri3ao digits inside the
 * GEMM instead of a separate slicing pass (less scratch, usually slower);
 * chunks_per_item: exact contraction chunks per work item of the persistent
 * GEMM (split-K granularity), 0 = fill whole waves.  Chosen per batch shape
 * by the package's autotuner. */
typedef struct {
    int fuse;
    int chunks_per_item;
} rt_tuning;

/* rt_ri_ov_k for many independent molecules of uneven sizes.  Each of the
 * three products (X = B C_occ, ov, K) of all molecules goes out as one grouped
 * persistent GEMM launch (split form, up to 48 molecules per launch) or one
 * grouped DFMA launch (float64 form, up to 64).  The call makes no host
 * synchronisation and can be captured in a CUDA graph (after a first,
 * uncaptured call has set the kernels' shared-memory limits). tuning may be NULL. */
rt_status rt_ri_ov_k_batched(const rt_ri_problem* probs, int nprob, int form, int nslices, const rt_tuning* tuning,
                             void* stream);

/* RI-J: w[P] = sum_{mu,nu} B^P[mu,nu] D[mu,nu] ("ip,ip->p", _einsum_02,
 * src/matrix/matrix_blas_lapack.rs:1293-1310 on the [nb*nb, naux] view of
 * ri.rs:309-316) and J = sum_P w[P] B^P.  w may be NULL. */
rt_status rt_ri_j(const double* B, const double* D, int nb, int naux, double* w, double* J, void* stream);

/* rt_ri_j for symmetric slabs and a symmetric D, the case of (mu nu|P) and of
 * a density matrix: reads only the entries mu <= nu of every B^P and of D (the
 * rest may hold anything) and forms each product once, w[P] as
 * sum_{mu<=nu} (2 - delta_{mu nu}) D[mu,nu] B^P[mu,nu] and J's upper triangle,
 * which it mirrors.  Both passes are bound by the float64 FMA rate, so this
 * takes about half the time of rt_ri_j.  No counterpart in the reference (its
 * ri3fn has the same symmetry; rt_ri_j follows its full contraction).
 * With RT_CHECK_SYMMETRY=1 in the environment it first compares every mirror
 * pair of B's first slab and of D, and 64 sampled pairs of every other slab;
 * a mismatch makes the next rt_sync_status return RT_ERR_INVALID_ARG. */
rt_status rt_ri_j_symmetric(const double* B, const double* D, int nb, int naux, double* w, double* J, void* stream);

/* Exchange energy E_x = -tr(D K) = -sum_{mu,nu} D[mu,nu] K[mu,nu], reduced in
 * float64 with a fixed-order tree.  Writes one double to ex_device. */
rt_status rt_ri_exchange_energy(const double* D, const double* K, int nb, double* ex_device, void* stream);

/* Eigen-decomposition of the symmetric n x n device matrix A (column-major;
 * only its lower triangle is read), replacing lapack_dsyev
 * (src/matrix/matrix_blas_lapack.rs:775-797, dsyev 'V', 'L'): eigenvalues in
 * ascending order into w[n] (device), orthonormal eigenvectors into the
 * columns of A.  Float64 throughout: Householder tridiagonalisation and the
 * accumulation of its reflectors on the device, the implicit QR iteration on
 * the tridiagonal on the host, its rotations applied on the device.  Each
 * eigenvector's largest-magnitude component is positive.  Synchronises
 * `stream`.  Scratch: about 3 n^2 doubles. */
rt_status rt_dsyev(int n, double* A, double* w, void* stream);

/* S^p of a symmetric n x n device matrix, replacing lapack_power
 * (src/matrix/matrix_blas_lapack.rs:1004-1064): with S = V diag(ev) V^T,
 *   out = sum over ev_i >= threshold of sqrt(ev_i)^p * sqrt(ev_i)^p v_i v_i^T
 * (eigenpairs below the threshold are dropped, as the reference zeroes their
 * columns).  n_nonsingular (host, may be NULL) receives the number kept.  The
 * final product out = E E^T runs in the float64 form (RT_FORM_FP64) or the
 * split form (RT_FORM_SPLIT, nslices 3..8); the eigensolver is float64.
 * Synchronises `stream`. */
rt_status rt_lapack_power(const double* S, int n, double p, double threshold, double* out, int* n_nonsingular,
                          int form, int nslices, void* stream);

/* The lowest num_orb eigenpairs of A x = lambda B x, replacing lapack_dspgvx
 * (src/matrix/matrix_blas_lapack.rs:1096-1147, dspgvx itype 1, 'V', 'I', 'U'):
 * A and B in packed upper storage (MatrixUpper: (i, j), i <= j, at
 * ap[i + j (j + 1) / 2]) on the device, B positive definite.  eigvec[n,
 * num_orb] receives B-orthonormal eigenvectors (x^T B x = 1), w[n] the num_orb
 * eigenvalues in ascending order followed by zeros, as the reference's vector
 * holds them.  Computed through B = U diag(b) U^T, X = U diag(b)^-1/2 and the
 * eigenvectors y of X^T A X (x = X y) rather than a Cholesky factor of B; the
 * three n x n products run in `form`.  Returns RT_ERR_INVALID_ARG when B is not
 * positive definite (the reference panics).  Synchronises `stream`. */
rt_status rt_dspgvx(const double* ap, const double* bp, int n, int num_orb, double* eigvec, double* w, int form,
                    int nslices, void* stream);

/* Inverse square root of a symmetric positive matrix by Newton-Schulz
 * iteration, _newton_schulz_inverse_square_root_v02
 * (src/matrix/matrix_blas_lapack.rs:1710-1778) with its per-stage iteration
 * _newton_schulz_inverse_square_root_lf (:1780-1932): the matrix is
 * normalised by its Frobenius norm; for each level shift in turn,
 *   X <- 0.5 X (3I - A X X)
 * runs from the previous stage's result until ||X_next - X||_F / n^2 <=
 * threshold, with the reference's mixing branches; a stage that fails is
 * retried with the mixing parameter halved (at most six times), after which
 * the stages stop.  The result is rescaled by ||S||_F^-1/2 into out[n, n].
 * S and out are device pointers; level_shift (n_level_shift >= 1 entries) is
 * host memory.  converged (may be NULL) receives the reference's flag; steps
 * (may be NULL) the number of X_next evaluations over all stages and retries
 * (three n x n products each).  form
 * RT_FORM_FP64, or RT_FORM_SPLIT (nslices 3..8) for the three products of a
 * step.  Synchronises `stream` once per step (the branches depend on norms). */
rt_status rt_newton_schulz_inv_sqrt(const double* S, int n, double threshold, double mix_parameter, int num_iter,
                                    const double* level_shift, int n_level_shift, int form, int nslices,
                                    double* out, int* converged, int* steps, void* stream);

/* ------------------------------------------------------------------------
 * Layout utilities (device pointers).  Blocks are given by 0-based starts
 * and lengths; a source and target that share memory behave as a Fortran
 * array assignment (the source is read in full before the target is written).
 * ------------------------------------------------------------------------ */

/* copy_mm (restmatr.f90:197-212; Rust matr_copy, src/external_libs/mod.rs:102-120):
 *   t_matr[tx:tx+x_len, ty:ty+y_len] = f_matr[fx:fx+x_len, fy:fy+y_len] */
rt_status rt_copy_mm(int x_len, int y_len, const double* f_matr, int f_x_len, int f_y_len, int f_x_start,
                     int f_y_start, double* t_matr, int t_x_len, int t_y_len, int t_x_start, int t_y_start,
                     void* stream);

/* copy_mr (restmatr.f90:215-238; Rust ri_copy_from_matr, mod.rs:145-165): a
 * matrix block [x1_len, x2_len] into the rank-3 tensor t_ri[X, Y, Z] at
 *   mode 0: t_ri[a, b, t_x3]   mode 1: t_ri[a, t_x3, b]   mode 2: t_ri[t_x3, a, b]
 * with a = t_x1_start.., b = t_x2_start...  Other modes: RT_ERR_INVALID_ARG
 * (the Fortran silently copies nothing). */
rt_status rt_copy_mr(int x1_len, int x2_len, const double* f_matr, int f_x_len, int f_y_len, int f_x1_start,
                     int f_x2_start, double* t_ri, int t_x_len, int t_y_len, int t_z_len, int t_x1_start,
                     int t_x2_start, int t_x3, int mode, void* stream);

/* copy_rm (restmatr.f90:237-264; Rust matr_copy_from_ri, mod.rs:123-140): the
 * reverse of copy_mr, from f_ri[X, Y, Z] (same modes) into a matrix block. */
rt_status rt_copy_rm(int x1_len, int x2_len, const double* f_ri, int f_x_len, int f_y_len, int f_z_len,
                     int f_x1_start, int f_x2_start, int f_x3, int mode, double* t_matr, int t_x_len, int t_y_len,
                     int t_x1_start, int t_x2_start, void* stream);

/* copy_rr (restmatr.f90:266-285; Rust ri_copy_from_ri, mod.rs:168-190): a
 * [x1_len, x2_len, x3_len] block between two rank-3 tensors. */
rt_status rt_copy_rr(int x1_len, int x2_len, int x3_len, const double* f_ri, int f_x1_len, int f_x2_len,
                     int f_x3_len, int f_x1_start, int f_x2_start, int f_x3_start, double* t_ri, int t_x1_len,
                     int t_x2_len, int t_x3_len, int t_x1_start, int t_x2_start, int t_x3_start, void* stream);

/* RIFull transposes (src/ri.rs:225-295): `in` is [i, j, k]; `order` names the
 * output's axes, e.g. "jik" -> [j, i, k] (transpose_jik), "jki", "kji", "ikj"
 * (any permutation of "ijk" is accepted):  out[.. in the named order ..] = in[a_i, a_j, a_k]. */
rt_status rt_ri_transpose(const double* in, int i, int j, int k, const char* order, double* out, void* stream);

/* rifull_to_matfull_symm (src/ri.rs:296-307, 330-341): [nao, nao, naux] ->
 * [nao (nao + 1) / 2, naux], keeping rows r <= column c of every slab, packed
 * column after column: out[c (c + 1) / 2 + r, P] = in[r, c, P]. */
rt_status rt_ri_pack_symm(const double* in, int nao, int naux, double* out, void* stream);

/* ------------------------------------------------------------------------
 * Response operator and Davidson solver.
 * ------------------------------------------------------------------------ */

/* (ia|jb) block M = B_ov B_ov^T, B_ov = [nov, naux] column-major (the (i,a,P)
 * output of rt_ri_ov_k viewed as [nocc*nvir, naux]); M = [nov, nov]. */
rt_status rt_ri_iajb(const double* Bov, long long nov, int naux, double* M, int form, int nslices, void* stream);

/* RI response operator on a block of vectors, A = diag(delta) + B_ov B_ov^T:
 * AX = delta .* X + B_ov (B_ov^T X), X and AX = [nov, nvec]. */
rt_status rt_ri_response_matvec(const double* Bov, const double* delta, long long nov, int naux, const double* X,
                                double* AX, int nvec, int form, int nslices, void* stream);

/* Matrix-vector product callback for the Davidson solver: ax[:, v] = A x[:, v]
 * for the nvec columns of x (device pointers, column-major, leading dimension
 * n), on `stream`.  It plays the role of the `a_x` closure of
 * davidson_solve (src/davidson.rs:48-53). */
typedef rt_status (*rt_matvec_fn)(const double* x, double* ax, int nvec, long long n, void* ctx, void* stream);

/* DavidsonParams (src/davidson.rs:28-46); defaults tol 1e-5, maxcyc 50,
 * maxspace 12, lindep 1e-14, nroots 3. */
typedef struct {
    double tol;
    int maxcyc;
    int maxspace;
    double lindep;
    int nroots;
} rt_davidson_params;

/* Lowest `nroots` eigenpairs of a symmetric operator, davidson_solve
 * (src/davidson.rs:48-266): one starting vector x0_1d, diagonal hdiag for the
 * preconditioner (both device, length n).  Outputs conv[nroots], e[nroots]
 * (host) and x_out[n, nroots] (device); `iterations` receives the cycle count
 * (may be NULL).  Vectors stay on the device; the subspace eigenproblem is
 * solved in float64 on the host. */
rt_status rt_davidson_solve(rt_matvec_fn a_x, void* ctx, const double* x0_1d, const double* hdiag, long long n,
                            const rt_davidson_params* params, int print_level, int* conv, double* e, double* x_out,
                            int* iterations, void* stream);

/* rt_davidson_solve on the RI response operator diag(delta) + B_ov B_ov^T.
 * The preconditioner uses the operator's exact diagonal,
 * delta[ia] + sum_P B_ov[ia, P]^2, formed on the device. */
rt_status rt_davidson_ri_response(const double* Bov, const double* delta, long long nov, int naux, int form,
                                  int nslices, const double* x0_1d, const rt_davidson_params* params, int print_level,
                                  int* conv, double* e, double* x_out, int* iterations, void* stream);

/* Fill B[nb, nb, naux] with the deterministic synthetic ri3ao tensor of
 * include/rt_synth.h (slabs P0..P0+nslab-1 of the full tensor, stored from B). */
rt_status rt_synth_ri3ao(uint64_t seed, int nb, int P0, int nslab, double* B, void* stream);

/* Fill d[nov] with the synthetic orbital-energy-difference diagonal of the
 * response problem (rt_delta_elem of include/rt_synth.h, uniform in [0.5, 3.0]). */
rt_status rt_synth_delta(uint64_t seed, long long nov, double* d, void* stream);

/* Fill M[nb, nb] with the N(0,1) matrix whose QR factor gives the synthetic
 * orbital coefficients (include/rt_synth.h, rt_coef_seed_elem). */
rt_status rt_synth_coef_seed(uint64_t seed, int nb, double* M, void* stream);

/* Host-pointer form of rt_ri_ov_k: copies C and B to the device, runs the
 * path, copies ov and K back, all on the given stream (synchronised on
 * return).  Host buffers may be pageable or pinned; pinned ri3ao slabs are
 * read by the SMs directly, pageable ones go through the copy engine. */
rt_status rt_ri_ov_k_host(const double* C, const double* B, int nb, int naux, int nocc, int nvir, double* ov,
                          double* K, int form, int nslices, void* stream);

/* Host-pointer form of rt_ri_ao2mo (the full transform ri3mo[P,p,q], P
 * fastest), pipelined over the host link: ri3ao slab blocks stream in while
 * the half-transform of the previous block runs, and ri3mo is produced in
 * blocks of q columns (contiguous in the P-fastest layout) whose copies back
 * overlap the next block's GEMM.  Host buffers may be pageable (a Rust Vec) or
 * pinned.  Every element equals rt_ri_ao2mo's on the same inputs.  Needs
 * about 2 nb^2 naux doubles of device scratch.  Synchronised on return.  The
 * body of the drop-in ri_ao2mo_f_ (restmatr.f90:158-194). */
rt_status rt_ri_ao2mo_host(const double* C, const double* B, double* ri3mo, int nb, int ns, int naux, int form,
                           int nslices, void* stream);

/* rt_ri_ov_k_host for symmetric ri3ao slabs (B^P_{mu,nu} = B^P_{nu,mu}, as the
 * three-centre integrals (mu nu|P) always are): only the upper triangle of each
 * slab crosses the host link and the lower triangle is mirrored on the device.
 * Page-locked B is read in place by a gather kernel (2 CTAs per SM, on a
 * high-priority stream); pageable B goes by 3-D copies of 32-column blocks.
 * The results are those of rt_ri_ov_k_host on the slabs symmetrised from their
 * upper triangles.  No counterpart in the reference (its ri_ao2mo_f reads the
 * full tensor).  With RT_CHECK_SYMMETRY=1 in the environment it first compares
 * every mirror pair of the first slab and 64 sampled pairs of every other slab
 * in host memory, and returns RT_ERR_INVALID_ARG on a mismatch. */
rt_status rt_ri_ov_k_host_symmetric(const double* C, const double* B, int nb, int naux, int nocc, int nvir,
                                    double* ov, double* K, int form, int nslices, void* stream);

/* ------------------------------------------------------------------------
 * Instrumentation.
 * ------------------------------------------------------------------------ */

/* Number of kernels this library has launched in the process so far. */
long long rt_launch_count(void);
/* Enable (1) or disable (0) per-kernel CUDA-event timing; either call clears
 * the records.  Kinds: 0 split-precision GEMM (flops = BF16 digit-pair
 * tensor operations), 1 digit slicing (bytes), 2 float64 GEMM (flops),
 * 3 RI-J streaming (bytes). */
void rt_profile_enable(int on);
/* Total event time, launch count and algorithmic work recorded for a kind
 * (synchronises the recorded events). */
rt_status rt_profile_get(int kind, double* total_ms, long long* launches, double* work);

/* ---- Testing hooks (no counterpart in the reference) ----
 * rt_debug_fail_alloc_after(n): the next n scratch allocations succeed and the
 * one after fails with RT_ERR_NO_MEMORY (n < 0: off).  Process-wide.
 * rt_debug_wait_timeout(cycles, stream): a one-thread kernel waits on a barrier
 * that nothing arrives at, for at most `cycles` clock cycles (<= 2e9), then sets
 * the device error word's timeout flag and returns normally; rt_sync_status()
 * then reports RT_ERR_TIMEOUT.  This is the library's bounded-wait path run out
 * on purpose; no device fault is raised.
 * rt_debug_chunk_bytes(bytes): bound on the scratch of one staged chunk of
 * y-slices in rt_special_dgemm_01 (default 8 GB; bytes <= 0 restores it), so
 * that small tensors can run through several chunks.  Process-wide. */
rt_status rt_debug_fail_alloc_after(long long n);
rt_status rt_debug_wait_timeout(long long cycles, void* stream);
rt_status rt_debug_chunk_bytes(long long bytes);
/* rt_debug_symeig(n, a, w, z): the Davidson subspace eigensolver on a host
 * column-major symmetric matrix a[n, n]: eigenvalues ascending in w[n],
 * eigenvectors in the columns of z[n, n], each with its largest-magnitude
 * component positive.  Host code only; callable without a GPU. */
rt_status rt_debug_symeig(int n, const double* a, double* w, double* z);

#ifdef __cplusplus
}
#endif

#endif /* REST_TENSORS_GB300_H */
