/*
 * oracle.c - CPU restatement of rest_tensors' dense RI contraction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is loaded by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, and by
 * nothing in the product library.  It restates the reference's algorithms on
 * the host and calls OpenBLAS/LAPACK by their exported names, exactly as the
 * reference reaches BLAS from Fortran (src/external_libs/restmatr.f90) and
 * from Rust (src/matrix/matrix_blas_lapack.rs).  The BLAS is the OpenBLAS
 * build bundled with scipy (LP64, symbols prefixed "scipy_"), opened with
 * dlopen at run time; its path is passed to oracle_init().
 *
 * Parity pins: the GEMM seam (general_dgemm_f, _dgemm) and the LAPACK
 * eigen-solver are pinned to the reference's doctest vectors
 * (src/external_libs/mod.rs:30-59, src/matrix/matrix_blas_lapack.rs:78-120,
 * 285-318).  The RI contractions themselves have no reference test; they are
 * cross-checked against numpy einsum and analytic identities in tests/.
 */
#define _GNU_SOURCE
#include <dlfcn.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../include/rt_synth.h"

typedef void (*dgemm_fn)(const char*, const char*, const int*, const int*, const int*,
                         const double*, const double*, const int*, const double*, const int*,
                         const double*, double*, const int*);
typedef void (*dgemv_fn)(const char*, const int*, const int*, const double*, const double*,
                         const int*, const double*, const int*, const double*, double*, const int*);
typedef void (*dspevx_fn)(const char*, const char*, const char*, const int*, double*,
                          const double*, const double*, const int*, const int*, const double*,
                          int*, double*, double*, const int*, double*, int*, int*, int*);
typedef void (*dsyev_fn)(const char*, const char*, const int*, double*, const int*, double*,
                         double*, const int*, int*);
typedef void (*dspgvx_fn)(const int*, const char*, const char*, const char*, const int*, double*, double*,
                          const double*, const double*, const int*, const int*, const double*, int*, double*,
                          double*, const int*, double*, int*, int*, int*);
typedef void (*setthreads_fn)(int);
typedef int (*getthreads_fn)(void);

static dgemm_fn p_dgemm;
static dgemv_fn p_dgemv;
static dspevx_fn p_dspevx;
static dsyev_fn p_dsyev;
static dspgvx_fn p_dspgvx;
static setthreads_fn p_set_threads;
static getthreads_fn p_get_threads;

static void* sym(void* h, const char* a, const char* b) {
    void* p = dlsym(h, a);
    if (!p && b) p = dlsym(h, b);
    return p;
}

/* Returns 0 on success, a negative code naming the missing piece otherwise. */
int oracle_init(const char* openblas_path) {
    void* h = dlopen(openblas_path, RTLD_NOW | RTLD_LOCAL);
    if (!h) return -1;
    p_dgemm = (dgemm_fn)sym(h, "scipy_dgemm_", "dgemm_");
    p_dgemv = (dgemv_fn)sym(h, "scipy_dgemv_", "dgemv_");
    p_dspevx = (dspevx_fn)sym(h, "scipy_dspevx_", "dspevx_");
    p_dsyev = (dsyev_fn)sym(h, "scipy_dsyev_", "dsyev_");
    p_dspgvx = (dspgvx_fn)sym(h, "scipy_dspgvx_", "dspgvx_");
    p_set_threads = (setthreads_fn)sym(h, "scipy_openblas_set_num_threads", "openblas_set_num_threads");
    p_get_threads = (getthreads_fn)sym(h, "scipy_openblas_get_num_threads", "openblas_get_num_threads");
    if (!p_dgemm || !p_dgemv) return -2;
    if (!p_dspevx || !p_dsyev || !p_dspgvx) return -3;
    return 0;
}

void oracle_set_threads(int n) { if (p_set_threads) p_set_threads(n); }
int oracle_get_threads(void) { return p_get_threads ? p_get_threads() : 1; }

/* ------------------------------------------------------------------------ */
/* GEMM seam                                                                 */
/* ------------------------------------------------------------------------ */

/* Column-major dgemm passthrough (matrix_blas_lapack.rs:739-774 lapack_dgemm
 * passes lda = m|k by op, ldb = k|n by op, ldc = m). */
void oracle_dgemm(char opa, char opb, int m, int n, int k, double alpha, const double* a, int lda,
                  const double* b, int ldb, double beta, double* c, int ldc) {
    if (m <= 0 || n <= 0) return;
    p_dgemm(&opa, &opb, &m, &n, &k, &alpha, a, &lda, b, &ldb, &beta, c, &ldc);
}

static void copy_block_in(const double* m, int rows, int r0, int nr, int c0, int nc, double* out) {
    for (int j = 0; j < nc; ++j)
        memcpy(out + (size_t)j * nr, m + (size_t)(c0 + j) * rows + r0, sizeof(double) * (size_t)nr);
}

/*
 * restmatr.f90:63-107 general_dgemm_f.  The Fortran passes array sections,
 * which gfortran materialises as contiguous copy-in/copy-out temporaries; the
 * leading dimensions follow the Fortran exactly:
 *   opa=='N' -> k = len_column_a, lda = len_row_c ; else k = len_row_a, lda = len_row_a
 *   opb=='N' -> ldb = len_row_b                  ; else ldb = len_column_c
 *   ldc = len_row_c
 * The sizes rows_x/columns_x are the full matrix shapes (column-major).
 */
void oracle_general_dgemm_f(const double* a, int rows_a, int columns_a, int start_row_a, int len_row_a,
                            int start_column_a, int len_column_a, char opa,
                            const double* b, int rows_b, int columns_b, int start_row_b, int len_row_b,
                            int start_column_b, int len_column_b, char opb,
                            double* c, int rows_c, int columns_c, int start_row_c, int len_row_c,
                            int start_column_c, int len_column_c, double alpha, double beta) {
    (void)columns_a; (void)columns_b; (void)columns_c;
    int k, lda, ldb;
    if (opa == 'N') { k = len_column_a; lda = len_row_c; }
    else { k = len_row_a; lda = len_row_a; }
    if (opb == 'N') ldb = len_row_b;
    else ldb = len_column_c;
    double* ta = (double*)malloc(sizeof(double) * (size_t)len_row_a * (size_t)len_column_a + 8);
    double* tb = (double*)malloc(sizeof(double) * (size_t)len_row_b * (size_t)len_column_b + 8);
    double* tc = (double*)malloc(sizeof(double) * (size_t)len_row_c * (size_t)len_column_c + 8);
    copy_block_in(a, rows_a, start_row_a, len_row_a, start_column_a, len_column_a, ta);
    copy_block_in(b, rows_b, start_row_b, len_row_b, start_column_b, len_column_b, tb);
    copy_block_in(c, rows_c, start_row_c, len_row_c, start_column_c, len_column_c, tc);
    int ldc = len_row_c;
    p_dgemm(&opa, &opb, &len_row_c, &len_column_c, &k, &alpha, ta, &lda, tb, &ldb, &beta, tc, &ldc);
    for (int j = 0; j < len_column_c; ++j)
        memcpy(c + (size_t)(start_column_c + j) * rows_c + start_row_c, tc + (size_t)j * len_row_c,
               sizeof(double) * (size_t)len_row_c);
    free(ta); free(tb); free(tc);
}

/* ------------------------------------------------------------------------ */
/* AO -> MO transform                                                        */
/* ------------------------------------------------------------------------ */

/*
 * restmatr.f90:158-194 ri_ao2mo_f (called from src/ri.rs:382-408 ao2mo_v02).
 *   ri3mo(:,:,:) = 0
 *   do P = 1, naux
 *     tmp(nb,ns)     = ri3fn(:,:,P) * eigenvector          dgemm('N','N',nb,ns,nb)
 *     ri3mo(P,:,:)   = eigenvector^T * tmp                 dgemm('T','N',ns,ns,nb)
 * ri3mo is [naux, ns, ns] column-major (P fastest).  The Fortran passes
 * ldc = num_basis for the ns x ns section temporary, which is only valid when
 * ns == nb; this restatement uses the temporary's true leading dimension ns,
 * i.e. the intended mathematics, and is identical to the Fortran at ns == nb.
 * P0/P1 restrict the loop to a slab range (a bounded CPU sample).
 */
void oracle_ri_ao2mo_range(const double* eigenvector, const double* ri3fn, double* ri3mo, int ns, int nb,
                           int naux, int P0, int P1) {
    size_t nb2 = (size_t)nb * (size_t)nb;
    double* tmp = (double*)calloc((size_t)nb * (size_t)ns + 8, sizeof(double));
    double* sec = (double*)calloc((size_t)ns * (size_t)ns + 8, sizeof(double));
    for (size_t i = 0; i < (size_t)naux * (size_t)ns * (size_t)ns; ++i) ri3mo[i] = 0.0;
    for (int P = P0; P < P1; ++P) {
        oracle_dgemm('N', 'N', nb, ns, nb, 1.0, ri3fn + (size_t)P * nb2, nb, eigenvector, nb, 0.0, tmp, nb);
        oracle_dgemm('T', 'N', ns, ns, nb, 1.0, eigenvector, nb, tmp, nb, 0.0, sec, ns);
        for (int q = 0; q < ns; ++q)
            for (int p = 0; p < ns; ++p)
                ri3mo[(size_t)P + (size_t)naux * ((size_t)p + (size_t)ns * q)] = sec[p + (size_t)ns * q];
    }
    free(tmp); free(sec);
}

void oracle_ri_ao2mo_f(const double* eigenvector, const double* ri3fn, double* ri3mo, int ns, int nb, int naux) {
    oracle_ri_ao2mo_range(eigenvector, ri3fn, ri3mo, ns, nb, naux, 0, naux);
}

/*
 * Occupied-virtual transform plus RI-K, composed the way ri_ao2mo_f composes
 * its two dgemms (restmatr.f90:183-188), with C = [C_occ | C_vir]:
 *   X^P      = B^P C_occ                  dgemm('N','N', nb, nocc, nb)
 *   ov(:,:,P)= X^P^T C_vir  -> (i,a,P)    dgemm('T','N', nocc, nvir, nb)
 *   K       += X^P X^P^T                  dgemm('N','T', nb, nb, nocc, beta=1)
 * ov is [nocc, nvir, naux] column-major (i fastest); K is [nb, nb].
 * Slabs P0..P1 only (the rest of ov is left untouched; K sums the range).
 */
void oracle_ri_ov_k_range(const double* C, const double* B, int nb, int naux, int nocc, int nvir, double* ov,
                          double* K, int P0, int P1) {
    (void)naux;
    size_t nb2 = (size_t)nb * (size_t)nb;
    double* X = (double*)calloc((size_t)nb * (size_t)nocc + 8, sizeof(double));
    for (size_t i = 0; i < nb2; ++i) K[i] = 0.0;
    const double* Cvir = C + (size_t)nb * (size_t)nocc;
    for (int P = P0; P < P1; ++P) {
        oracle_dgemm('N', 'N', nb, nocc, nb, 1.0, B + (size_t)P * nb2, nb, C, nb, 0.0, X, nb);
        if (nvir > 0)
            oracle_dgemm('T', 'N', nocc, nvir, nb, 1.0, X, nb, Cvir, nb, 0.0,
                         ov + (size_t)P * (size_t)nocc * (size_t)nvir, nocc);
        oracle_dgemm('N', 'T', nb, nb, nocc, 1.0, X, nb, X, nb, 1.0, K, nb);
    }
    free(X);
}

void oracle_ri_ov_k(const double* C, const double* B, int nb, int naux, int nocc, int nvir, double* ov, double* K) {
    oracle_ri_ov_k_range(C, B, nb, naux, nocc, nvir, ov, K, 0, naux);
}

/*
 * RI-J.  w_P = sum_{mu,nu} B^P_{mu nu} D_{mu nu} is _einsum_02 ("ip,ip->p",
 * matrix_blas_lapack.rs:1293-1310) on the [nb*nb, naux] view of RIFull
 * (ri.rs:309-316), written as a dgemv 'T'; J = sum_P w_P B^P is the matching
 * dgemv 'N' (matrix_blas_lapack.rs:38-70 _dgemv).
 */
void oracle_ri_j(const double* B, const double* D, int nb, int naux, double* w, double* J) {
    int n2 = nb * nb, one = 1;
    double a = 1.0, z = 0.0;
    p_dgemv("T", &n2, &naux, &a, B, &n2, D, &one, &z, w, &one);
    p_dgemv("N", &n2, &naux, &a, B, &n2, w, &one, &z, J, &one);
}

/* E_x = -tr(D K) = -sum_P ||C_occ^T X^P||_F^2 (closed shell, D = C_occ C_occ^T).
 * Summed with pairwise blocks in long double so the checker's own rounding
 * stays far below the tolerances it is used to judge. */
double oracle_exchange_energy(const double* D, const double* K, int nb) {
    long double s = 0.0L;
    size_t n = (size_t)nb * (size_t)nb;
    for (size_t i = 0; i < n; ++i) s += (long double)D[i] * (long double)K[i];
    return -(double)s;
}

/* (ia|jb) block M = Bov Bov^T with Bov = [nov, naux] column-major ((i,a,P) layout). */
void oracle_iajb(const double* Bov, int nov, int naux, double* M) {
    oracle_dgemm('N', 'T', nov, nov, naux, 1.0, Bov, nov, Bov, nov, 0.0, M, nov);
}

/* Response-matrix product AX = diag(delta) X + Bov (Bov^T X), X = [nov, nvec]. */
void oracle_response_matvec(const double* Bov, const double* delta, int nov, int naux, const double* X, double* AX,
                            int nvec) {
    double* T = (double*)calloc((size_t)naux * (size_t)nvec + 8, sizeof(double));
    oracle_dgemm('T', 'N', naux, nvec, nov, 1.0, Bov, nov, X, nov, 0.0, T, naux);
    for (int v = 0; v < nvec; ++v)
        for (int i = 0; i < nov; ++i) AX[(size_t)v * nov + i] = delta[i] * X[(size_t)v * nov + i];
    oracle_dgemm('N', 'N', nov, nvec, naux, 1.0, Bov, nov, T, naux, 1.0, AX, nov);
    free(T);
}

/* ------------------------------------------------------------------------ */
/* LAPACK seam                                                               */
/* ------------------------------------------------------------------------ */

/*
 * matrix_blas_lapack.rs:1075-1095 lapack_dspevx: packed upper triangle,
 * jobz='V', range='A', uplo='U', abstol = SAFE_MINIMUM = 1e-16 (lib.rs:99).
 * ap has n(n+1)/2 entries and is overwritten; w[n], z[n*n].  Returns info.
 */
int oracle_dspevx_packed(int n, double* ap, double* w, double* z, int* nfound) {
    double vl = 0.0, vu = 0.0, abstol = 1.0e-16;
    int il = 0, iu = 0, info = 0, ldz = n > 0 ? n : 1;
    double* work = (double*)calloc((size_t)8 * (size_t)n + 8, sizeof(double));
    int* iwork = (int*)calloc((size_t)5 * (size_t)n + 8, sizeof(int));
    int* ifail = (int*)calloc((size_t)n + 8, sizeof(int));
    p_dspevx("V", "A", "U", &n, ap, &vl, &vu, &il, &iu, &abstol, nfound, w, z, &ldz, work, iwork, ifail, &info);
    free(work); free(iwork); free(ifail);
    return info;
}

/* matrix_blas_lapack.rs:319-348 _dsyev: jobz, uplo='L', lwork = 4n. */
int oracle_dsyev(char jobz, int n, double* a, double* w) {
    int lwork = 4 * n > 1 ? 4 * n : 1, info = 0;
    double* work = (double*)calloc((size_t)lwork + 8, sizeof(double));
    p_dsyev(&jobz, "L", &n, a, &n, w, work, &lwork, &info);
    free(work);
    return info;
}

/*
 * matrix_blas_lapack.rs:1004-1064 lapack_power: om = -S; dsyev('V','L') on om
 * (:1012, through lapack_dsyev :775-797, lwork 4n); the eigenvalues negated back
 * (largest first); columns i with ev_i >= threshold scaled by sqrt(ev_i)^p, the
 * others zeroed (:1042-1052); out = E E^T by dgemm('N','T') (:1056-1060).
 * n_nonsingular receives the number of eigenvalues >= threshold.  Returns the
 * dsyev info.
 */
int oracle_lapack_power(int n, const double* S, double p, double threshold, double* out, int* n_nonsingular) {
    const size_t nn = (size_t)n * (size_t)n;
    double* om = (double*)malloc(sizeof(double) * nn + 8);
    double* ev = (double*)malloc(sizeof(double) * (size_t)n + 8);
    for (size_t i = 0; i < nn; ++i) om[i] = -S[i];
    const int info = oracle_dsyev('V', n, om, ev);
    int kept = 0;
    for (int i = 0; i < n; ++i) {
        ev[i] = -ev[i];
        if (ev[i] >= threshold) ++kept;
    }
    for (int i = 0; i < n; ++i) {
        double* col = om + (size_t)i * n;
        if (i < kept) {
            const double f = pow(sqrt(ev[i]), p);
            for (int r = 0; r < n; ++r) col[r] *= f;
        } else {
            for (int r = 0; r < n; ++r) col[r] = 0.0;
        }
    }
    const double one = 1.0, zero = 0.0;
    p_dgemm("N", "T", &n, &n, &n, &one, om, &n, om, &n, &zero, out, &n);
    if (n_nonsingular) *n_nonsingular = kept;
    free(om); free(ev);
    return info;
}

/*
 * matrix_blas_lapack.rs:1096-1147 lapack_dspgvx: dspgvx(itype 1, 'V', 'I', 'U',
 * n, a, b, vl 0, vu 0, il 1, iu num_orb, abstol SAFE_MINIMUM = 1e-16 (lib.rs:99),
 * m, w, z, ldz n, work 8n, iwork 5n, ifail n) on packed upper copies of A and B.
 * z receives n x num_orb eigenvectors (the reference's [ndim, num_orb] view of
 * its n x n buffer), w all n entries (only the first m are set by LAPACK; the
 * rest stay 0 as in the reference's zero-initialised vector).  Returns info;
 * m_out receives m.
 */
int oracle_dspgvx(int n, const double* ap, const double* bp, int num_orb, double* z, double* w, int* m_out) {
    const size_t np = (size_t)n * (size_t)(n + 1) / 2;
    double* a = (double*)malloc(sizeof(double) * np + 8);
    double* b = (double*)malloc(sizeof(double) * np + 8);
    double* zz = (double*)calloc((size_t)n * (size_t)n + 8, sizeof(double));
    double* work = (double*)calloc((size_t)8 * (size_t)n + 8, sizeof(double));
    int* iwork = (int*)calloc((size_t)5 * (size_t)n + 8, sizeof(int));
    int* ifail = (int*)calloc((size_t)n + 8, sizeof(int));
    memcpy(a, ap, sizeof(double) * np);
    memcpy(b, bp, sizeof(double) * np);
    for (int i = 0; i < n; ++i) w[i] = 0.0;
    const int itype = 1, il = 1, iu = num_orb, ldz = n;
    const double vl = 0.0, vu = 0.0, abstol = 1.0e-16;
    int m = 0, info = 0;
    p_dspgvx(&itype, "V", "I", "U", &n, a, b, &vl, &vu, &il, &iu, &abstol, &m, w, zz, &ldz, work, iwork, ifail,
             &info);
    memcpy(z, zz, sizeof(double) * (size_t)n * (size_t)num_orb);
    if (m_out) *m_out = m;
    free(a); free(b); free(zz); free(work); free(iwork); free(ifail);
    return info;
}

/*
 * restmatr.f90:111-154 special_dgemm_f_01 (the O_V * V^{-1/2} step of the
 * ri3fn preparation).  For i_state = 1..y_a (i_y_a is never read) the Fortran
 * copies the section T = ten3_a(sx+1:sx+lx, i_state, sz+1:sz+lz) into
 * matr_c, calls
 *   dgemm('N','N', lx, len_column_b, lz, alpha, matr_c, lx,
 *         matr_b(section), lz, beta, matr_c, lx)
 * and copies matr_c back into the same section.  matr_b's section reaches
 * dgemm as a gfortran copy-in temporary with leading dimension lz.  The
 * Fortran passes matr_c as both A and C, which BLAS does not define; this
 * restatement gives dgemm a separate copy of T as A, which is the product
 * the arguments describe.
 */
void oracle_special_dgemm_f_01(double* ten3_a, int x_a, int y_a, int z_a, int start_x_a, int len_x_a,
                               int start_z_a, int len_z_a, const double* matr_b, int rows_b, int columns_b,
                               int start_row_b, int len_row_b, int start_column_b, int len_column_b,
                               double alpha, double beta) {
    (void)z_a; (void)columns_b;
    const int lx = len_x_a, lz = len_z_a, n = len_column_b;
    if (lx <= 0 || lz <= 0 || n <= 0) return;
    const size_t xy = (size_t)x_a * (size_t)y_a;
    double* ta = (double*)malloc(sizeof(double) * (size_t)lx * (size_t)lz);
    double* tc = (double*)malloc(sizeof(double) * (size_t)lx * (size_t)n);
    double* tb = (double*)malloc(sizeof(double) * (size_t)len_row_b * (size_t)len_column_b);
    copy_block_in(matr_b, rows_b, start_row_b, len_row_b, start_column_b, len_column_b, tb);
    for (int i = 0; i < y_a; ++i) {
        for (int z = 0; z < lz; ++z)
            memcpy(ta + (size_t)z * lx, ten3_a + (size_t)start_x_a + (size_t)i * x_a + (size_t)(start_z_a + z) * xy,
                   sizeof(double) * (size_t)lx);
        for (int z = 0; z < n; ++z) memcpy(tc + (size_t)z * lx, ta + (size_t)z * lx, sizeof(double) * (size_t)lx);
        int m = lx, k = lz, ld = lx, ldb = lz;
        p_dgemm("N", "N", &m, &n, &k, &alpha, ta, &ld, tb, &ldb, &beta, tc, &ld);
        for (int z = 0; z < n; ++z)
            memcpy(ten3_a + (size_t)start_x_a + (size_t)i * x_a + (size_t)(start_z_a + z) * xy, tc + (size_t)z * lx,
                   sizeof(double) * (size_t)lx);
    }
    free(ta); free(tb); free(tc);
}

/* ------------------------------------------------------------------------ */
/* Synthetic inputs (same formulas as the device generator)                  */
/* ------------------------------------------------------------------------ */

void oracle_synth_ri3ao(uint64_t seed, int nb, int naux, int P0, int P1, double* B) {
    size_t nb2 = (size_t)nb * (size_t)nb;
    #pragma omp parallel for schedule(static)
    for (int P = P0; P < P1; ++P)
        for (int nu = 0; nu < nb; ++nu)
            for (int mu = 0; mu < nb; ++mu)
                B[(size_t)(P - P0) * nb2 + (size_t)nu * nb + mu] = rt_ri3ao_elem(seed, P, mu, nu);
    (void)naux;
}

void oracle_synth_coef_seed(uint64_t seed, int nb, double* M) {
    for (int c = 0; c < nb; ++c)
        for (int r = 0; r < nb; ++r) M[(size_t)c * nb + r] = rt_coef_seed_elem(seed, r, c);
}

void oracle_synth_delta(uint64_t seed, int64_t nov, double* d) {
    for (int64_t i = 0; i < nov; ++i) d[i] = rt_delta_elem(seed, i);
}
