// capi.cu - the exported C ABI: the reference's Fortran seam (drop-in, host
// pointers) and the rt_* device-pointer API, composed from the float64 and
// split-precision GEMM services.
#include <stdlib.h>
#include <string.h>
#include <strings.h>

#include <algorithm>
#include <atomic>
#include <vector>

#include "rt_internal.cuh"

namespace rt {


rt_status ri_j_fp64(const double* B, const double* D, int nb, int naux, double* w, double* J, cudaStream_t stream);
rt_status ri_j_fp64_symmetric(const double* B, const double* D, int nb, int naux, double* w, double* J,
                              cudaStream_t stream);
rt_status exchange_energy(const double* D, const double* K, int nb, double* out, cudaStream_t stream);
rt_status synth_ri3ao(uint64_t seed, int nb, int P0, int nslab, double* B, cudaStream_t stream);
rt_status synth_coef_seed(uint64_t seed, int nb, double* M, cudaStream_t stream);
rt_status synth_delta(uint64_t seed, int64_t nov, double* d, cudaStream_t stream);
rt_status ri_ao2mo_fp64(const double* C, const double* B, double* R, int nb, int ns, int naux, cudaStream_t stream);
rt_status ri_ov_k_fp64(const double* C, const double* B, int nb, int naux, int nocc, int nvir, double* ov,
                       double* K, cudaStream_t stream);

namespace {

// Slabs per split-precision block so that the BF16 digit planes of one block
// stay within ~16 GB of scratch.
int64_t split_block(int64_t nb, int64_t naux, int S) {
    const int64_t kpad = (nb + 31) / 32 * 32;
    const int64_t per = nb * kpad * 2 * S;
    int64_t blk = ((int64_t)16 << 30) / std::max<int64_t>(per, 1);
    return std::max<int64_t>(1, std::min<int64_t>(blk, naux));
}

// chunks_per_item for "the whole contraction range in one work item".
constexpr int kWholeRange = 1 << 30;

// The two split-form products of the full transform.  Neither splits its
// contraction, so a CTA's int64 range guard depends only on nb and every
// element is the same however the slabs or columns are blocked.
// T^P = B^P C over slabs [0, np) of B:  A(m=(mu,P), k=nu) = B[mu + nb nu + nb^2 P],
// B(n=p, k=nu) = C[nu + nb p],  T[mu + nb p + nb ns P].
OzGemm t_product(const double* C, const double* B, int nb, int ns, int64_t np, double* T, int S) {
    OzGemm g;
    g.K = nb;
    g.A.p = B; g.A.rows = (int64_t)nb * np; g.A.div = nb;
    g.A.s0 = 1; g.A.s1 = (int64_t)nb * nb; g.A.sk = nb;
    g.B.p = C; g.B.rows = ns; g.B.s0 = nb; g.B.sk = 1;
    g.C.p = T; g.C.md = nb; g.C.ms0 = 1; g.C.ms1 = (int64_t)nb * ns; g.C.ns0 = nb;
    g.nslices = S;
    g.chunks_per_item = kWholeRange;
    return g;
}

// R[P + naux p + naux ns q] = sum_mu C[mu,p] T^P[mu,q] for nq columns q of T (Tq = T + nb q0) over np
// slabs:  A(m=(q,P), k=mu) = Tq[mu + nb q + nb ns P],  B(n=p, k=mu) = C[mu + nb p],  output from Rq =
// R + P0 + naux ns q0.
OzGemm r_product(const double* C, const double* Tq, int nb, int ns, int64_t nq, int64_t np, int naux, double* Rq,
                 int S) {
    OzGemm g;
    g.K = nb;
    g.A.p = Tq; g.A.rows = nq * np; g.A.div = nq;
    g.A.s0 = nb; g.A.s1 = (int64_t)nb * ns; g.A.sk = 1;
    g.B.p = C; g.B.rows = ns; g.B.s0 = nb; g.B.sk = 1;
    g.C.p = Rq; g.C.md = nq; g.C.ms0 = (int64_t)naux * ns; g.C.ms1 = 1; g.C.ns0 = naux;
    g.nslices = S;
    g.chunks_per_item = kWholeRange;
    return g;
}

rt_status ri_ao2mo_split(const double* C, const double* B, double* R, int nb, int ns, int naux, int S,
                         cudaStream_t stream) {
    const int64_t blk = split_block(nb, naux, S);
    const int64_t per = (int64_t)nb * ns;
    ScratchBuf xb;
    RT_TRY(scratch_alloc(xb, sizeof(double) * (size_t)(per * blk), stream));
    double* T = xb.as<double>();
    for (int64_t P0 = 0; P0 < naux; P0 += blk) {
        const int64_t np = std::min<int64_t>(blk, naux - P0);
        RT_TRY(oz_gemm(t_product(C, B + P0 * (int64_t)nb * nb, nb, ns, np, T, S), stream));
        RT_TRY(oz_gemm(r_product(C, T, nb, ns, ns, np, naux, R + P0, S), stream));
    }
    return RT_OK;
}

// Half-transform and ov block for slabs [P0, P0 + np) of B (B already offset to slab P0):
//   X^P = B^P C_occ  ->  X[mu + nb i + nb nocc P],   ov[i,a,P] = (X^P^T C_vir)[i,a].

// The three split-form products of the ov + RI-K path.
// X^P = B^P C_occ:  A(m=(mu,P), k=nu) = B[mu + nb nu + nb^2 P], B(n=i, k=nu) = C[nu + nb i].
// No split-K for the two transform products: a CTA's int64 range guard
// depends on the terms it sums, so results then do not depend on how the
// slabs are blocked (the host entry streams them in blocks of any size).
OzGemm x_product(const double* C, const double* B, int nb, int64_t np, int nocc, double* X, int S) {
    const int64_t per = (int64_t)nb * nocc;
    OzGemm g;
    g.K = nb;
    g.A.p = B; g.A.rows = (int64_t)nb * np; g.A.div = nb;
    g.A.s0 = 1; g.A.s1 = (int64_t)nb * nb; g.A.sk = nb;
    g.B.p = C; g.B.rows = nocc; g.B.s0 = nb; g.B.sk = 1;
    g.C.p = X; g.C.md = nb; g.C.ms0 = 1; g.C.ms1 = per; g.C.ns0 = nb;
    g.nslices = S;
    g.chunks_per_item = kWholeRange;
    return g;
}

// ov^P = X^P^T C_vir:  A(m=(i,P), k=mu) = X[mu + nb m], B(n=a, k=mu) = C_vir[mu + nb a].
OzGemm ov_product(const double* C, int nb, int64_t np, int nocc, int nvir, const double* X, double* ov, int S) {
    const int64_t per = (int64_t)nb * nocc;
    OzGemm g;
    g.K = nb;
    g.A.p = X; g.A.rows = (int64_t)nocc * np; g.A.s0 = nb; g.A.sk = 1;
    g.B.p = C + per; g.B.rows = nvir; g.B.s0 = nb; g.B.sk = 1;
    g.C.p = ov; g.C.md = nocc; g.C.ms0 = 1; g.C.ms1 = (int64_t)nocc * nvir; g.C.ns0 = nocc;
    g.nslices = S;
    g.chunks_per_item = kWholeRange;
    return g;
}

// K = X X^T over k = (i, P):  A(m=mu, k) = X[mu + nb k], symmetric, B = A.
OzGemm k_product(const double* X, int nb, int nocc, int naux, double* K, int S) {
    OzGemm g;
    g.K = (int64_t)nocc * naux;
    g.A.p = X; g.A.rows = nb; g.A.s0 = 1; g.A.sk = nb;
    g.B = g.A;
    g.b_is_a = true;
    g.symmetric = true;
    g.C.p = K; g.C.ms0 = 1; g.C.ns0 = nb;
    g.nslices = S;
    return g;
}

rt_status ri_ov_block(const double* C, const double* B, int nb, int64_t np, int nocc, int nvir, double* X,
                      double* ov, int form, int S, cudaStream_t stream) {
    const int64_t per = (int64_t)nb * nocc;
    if (form == RT_FORM_FP64) {
        GemmF64 g1;
        g1.opa = 'N'; g1.opb = 'N'; g1.m = nb; g1.n = nocc; g1.k = nb;
        g1.A = B; g1.lda = nb; g1.sA = (int64_t)nb * nb;
        g1.B = C; g1.ldb = nb; g1.sB = 0;
        g1.C = X; g1.rsC = 1; g1.csC = nb; g1.bsC = per; g1.batch = np;
        RT_TRY(gemm_f64(g1, stream));
        if (ov && nvir > 0) {
            GemmF64 g2;
            g2.opa = 'T'; g2.opb = 'N'; g2.m = nocc; g2.n = nvir; g2.k = nb;
            g2.A = X; g2.lda = nb; g2.sA = per;
            g2.B = C + per; g2.ldb = nb; g2.sB = 0;
            g2.C = ov; g2.rsC = 1; g2.csC = nocc; g2.bsC = (int64_t)nocc * nvir; g2.batch = np;
            RT_TRY(gemm_f64(g2, stream));
        }
        return RT_OK;
    }
    RT_TRY(oz_gemm(x_product(C, B, nb, np, nocc, X, S), stream));
    if (ov && nvir > 0) RT_TRY(oz_gemm(ov_product(C, nb, np, nocc, nvir, X, ov, S), stream));
    return RT_OK;
}

// K[mu,nu] = sum_{(i,P)} X[mu + nb k] X[nu + nb k], k = i + nocc P.
rt_status ri_k_from_x(const double* X, int nb, int nocc, int naux, double* K, int form, int S, cudaStream_t stream) {
    const int64_t kdim = (int64_t)nocc * naux;
    if (form == RT_FORM_FP64) {
        GemmF64 g3;
        g3.opa = 'N'; g3.opb = 'T'; g3.m = nb; g3.n = nb; g3.k = kdim;
        g3.A = X; g3.lda = nb; g3.B = X; g3.ldb = nb;
        g3.C = K; g3.rsC = 1; g3.csC = nb;
        const int64_t tiles = ceil_div(nb, 64) * ceil_div(nb, 64);
        const int64_t want = (4 * sm_count() + tiles - 1) / tiles;
        g3.splitk = (int)std::max<int64_t>(1, std::min<int64_t>(want, kdim / 256));
        return gemm_f64(g3, stream);
    }
    return oz_gemm(k_product(X, nb, nocc, naux, K, S), stream);
}

rt_status ri_ov_k_split(const double* C, const double* B, int nb, int naux, int nocc, int nvir, double* ov,
                        double* K, int S, cudaStream_t stream) {
    const int64_t per = (int64_t)nb * nocc;
    ScratchBuf xb;
    RT_TRY(scratch_alloc(xb, sizeof(double) * (size_t)(per * naux), stream));
    double* X = xb.as<double>();
    const int64_t blk = split_block(nb, naux, S);
    for (int64_t P0 = 0; P0 < naux; P0 += blk) {
        const int64_t np = std::min<int64_t>(blk, naux - P0);
        RT_TRY(ri_ov_block(C, B + P0 * (int64_t)nb * nb, nb, np, nocc, nvir, X + P0 * per,
                           ov ? ov + P0 * (int64_t)nocc * nvir : nullptr, RT_FORM_SPLIT, S, stream));
    }
    if (K) RT_TRY(ri_k_from_x(X, nb, nocc, naux, K, RT_FORM_SPLIT, S, stream));
    return RT_OK;
}

// Scratch bound of one staged chunk of the ri3fn metric contraction
// (rt_debug_chunk_bytes lowers it for tests).
constexpr int64_t kMetricChunkBytes = (int64_t)8 << 30;
std::atomic<long long> g_chunk_bytes{kMetricChunkBytes};

// blk(xx, i, z) = alpha * blk(xx, i, z) + beta * S(xx, i, z) over the block
// [lx, ny, lz]; blk at xx + X i + XY z, S contiguous.
__global__ void __launch_bounds__(256) scale_add_block_kernel(double* __restrict__ blk,
                                                              const double* __restrict__ S, int64_t lx, int64_t ny,
                                                              int64_t lz, int64_t X, int64_t XY, double alpha,
                                                              double beta) {
    const int64_t nrow = ny * lz;
    for (int64_t r = blockIdx.y; r < nrow; r += gridDim.y) {
        const int64_t i = r % ny, z = r / ny;
        double* d = blk + i * X + z * XY;
        const double* src = S + r * lx;
        for (int64_t xx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; xx < lx;
             xx += (int64_t)gridDim.x * blockDim.x) {
            const double v = beta == 0.0 ? 0.0 : beta * src[xx];
            d[xx] = fma(alpha, d[xx], v);
        }
    }
}

// special_dgemm_f_01 (restmatr.f90:111-154) on device memory: for every
// y-slice of the rank-3 tensor T[X, Y, Z],
//   T[sx:sx+lx, y, sz:sz+lz] <- alpha * T[...] * M[srb:srb+lz, scb:scb+lz] + beta * T[...]
// Chunks of y-slices are staged in scratch (the product reads its left
// operand there), then written back in place: by the float64 GEMM with alpha
// and beta applied in its epilogue, or by the split GEMM followed by one
// scale-add pass when (alpha, beta) != (1, 0).
rt_status special_dgemm_01(double* T, int64_t X, int64_t Y, int64_t sx, int64_t lx, int64_t sz, int64_t lz,
                           const double* Mb, int64_t rows_b, int64_t srb, int64_t scb, double alpha, double beta,
                           int form, int S, cudaStream_t stream) {
    const int64_t XY = X * Y;
    const int64_t per_y = lx * lz;
    const int64_t chunk = g_chunk_bytes.load(std::memory_order_relaxed);
    const int64_t yc = std::max<int64_t>(1, std::min<int64_t>(Y, chunk / (8 * per_y)));
    ScratchBuf sb;
    RT_TRY(scratch_alloc(sb, sizeof(double) * (size_t)(per_y * yc), stream));
    double* St = sb.as<double>();
    const double* Msub = Mb + srb + rows_b * scb;
    for (int64_t y0 = 0; y0 < Y; y0 += yc) {
        const int64_t ny = std::min<int64_t>(yc, Y - y0);
        const int64_t M = lx * ny;
        double* blk = T + sx + X * y0 + XY * sz;
        Copy3 c;
        c.n[0] = lx; c.n[1] = ny; c.n[2] = lz;
        c.is[0] = 1; c.is[1] = X; c.is[2] = XY;
        c.os[0] = 1; c.os[1] = lx; c.os[2] = M;
        RT_TRY(strided_copy3(blk, St, c, stream));
        if (form == RT_FORM_FP64) {
            GemmF64 g;
            g.opa = 'N'; g.opb = 'N';
            g.m = M; g.n = lz; g.k = lz; g.alpha = alpha; g.beta = beta;
            g.A = St; g.lda = M;
            g.B = Msub; g.ldb = rows_b;
            g.C = blk; g.rsC = 1; g.csC = XY; g.c_md = lx; g.c_ms1 = X;
            RT_TRY(gemm_f64(g, stream));
        } else {
            // C(m, n) = sum_k A(m, k) B(n, k): A = the staged rows, B(n, k) = Msub(k, n).
            OzGemm g;
            g.K = lz;
            g.A.p = St; g.A.rows = M; g.A.s0 = 1; g.A.sk = M;
            g.B.p = Msub; g.B.rows = lz; g.B.s0 = rows_b; g.B.sk = 1;
            g.C.p = blk; g.C.md = lx; g.C.ms0 = 1; g.C.ms1 = X; g.C.ns0 = XY;
            g.nslices = S;
            RT_TRY(oz_gemm(g, stream));
            if (alpha != 1.0 || beta != 0.0) {
                const int64_t nrow = ny * lz;
                const unsigned gx = (unsigned)std::min<int64_t>((lx + 255) / 256, 8);
                const unsigned gy = (unsigned)std::min<int64_t>(nrow, 65535);
                scale_add_block_kernel<<<dim3(gx, gy), 256, 0, stream>>>(blk, St, lx, ny, lz, X, XY, alpha, beta);
                RT_TRY(check_launch("scale_add_block_kernel"));
            }
        }
    }
    return RT_OK;
}

bool valid_form(int form, int nslices) {
    return form == RT_FORM_FP64 || (form == RT_FORM_SPLIT && nslices >= 3 && nslices <= 8);
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

rt_status rt_dgemm(char opa, char opb, int m, int n, int k, double alpha, const double* A, int lda, const double* B,
                   int ldb, double beta, double* C, int ldc, void* stream) {
    NvtxRange nvtx_range("rt_dgemm");
    RT_REQUIRE(m >= 0 && n >= 0 && k >= 0, "rt_dgemm: negative dimension");
    RT_REQUIRE(opa == 'N' || opa == 'T' || opa == 'n' || opa == 't', "rt_dgemm: opa must be N or T");
    RT_REQUIRE(opb == 'N' || opb == 'T' || opb == 'n' || opb == 't', "rt_dgemm: opb must be N or T");
    const char oa = (opa == 'n') ? 'N' : (opa == 't' ? 'T' : opa);
    const char ob = (opb == 'n') ? 'N' : (opb == 't' ? 'T' : opb);
    RT_REQUIRE(lda >= std::max(1, oa == 'N' ? m : k), "rt_dgemm: lda too small");
    RT_REQUIRE(ldb >= std::max(1, ob == 'N' ? k : n), "rt_dgemm: ldb too small");
    RT_REQUIRE(ldc >= std::max(1, m), "rt_dgemm: ldc too small");
    GemmF64 g;
    g.opa = oa; g.opb = ob; g.m = m; g.n = n; g.k = k; g.alpha = alpha; g.beta = beta;
    g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.C = C; g.rsC = 1; g.csC = ldc;
    const int64_t tiles = ceil_div(m, 64) * ceil_div(n, 64);
    if (tiles < sm_count() && k >= 1024) g.splitk = (int)std::min<int64_t>(ceil_div(2 * sm_count(), tiles), k / 256);
    return gemm_f64(g, (cudaStream_t)stream);
}

rt_status rt_dgemm_split(char opa, char opb, int m, int n, int k, const double* A, int lda, const double* B, int ldb,
                         double* C, int ldc, int nslices, void* stream) {
    NvtxRange nvtx_range("rt_dgemm_split");
    RT_REQUIRE(m >= 0 && n >= 0 && k >= 0, "rt_dgemm_split: negative dimension");
    RT_REQUIRE(opa == 'N' || opa == 'T', "rt_dgemm_split: opa must be N or T");
    RT_REQUIRE(opb == 'N' || opb == 'T', "rt_dgemm_split: opb must be N or T");
    RT_REQUIRE(nslices >= 3 && nslices <= 8, "rt_dgemm_split: nslices must be in 3..8");
    RT_REQUIRE(lda >= std::max(1, opa == 'N' ? m : k), "rt_dgemm_split: lda too small");
    RT_REQUIRE(ldb >= std::max(1, opb == 'N' ? k : n), "rt_dgemm_split: ldb too small");
    RT_REQUIRE(ldc >= std::max(1, m), "rt_dgemm_split: ldc too small");
    cudaStream_t s = (cudaStream_t)stream;
    if (m == 0 || n == 0) return RT_OK;
    if (k == 0) {
        RT_CUDA_TRY(cudaMemset2DAsync(C, sizeof(double) * ldc, 0, sizeof(double) * m, n, s));
        return RT_OK;
    }
    OzGemm g;
    g.K = k;
    // C(i, j) = sum_k opA(i, k) opB(k, j), written as sum_k A'(i, k) B'(j, k)
    g.A.p = A; g.A.rows = m;
    if (opa == 'N') { g.A.s0 = 1; g.A.sk = lda; } else { g.A.s0 = lda; g.A.sk = 1; }
    g.B.p = B; g.B.rows = n;
    if (opb == 'N') { g.B.s0 = ldb; g.B.sk = 1; } else { g.B.s0 = 1; g.B.sk = ldb; }
    g.C.p = C; g.C.ms0 = 1; g.C.ns0 = ldc;
    g.nslices = nslices;
    // A * A^T (same matrix on both sides): slice once and compute one triangle.
    if (A == B && opa != opb && lda == ldb && m == n) {
        g.B = g.A;
        g.b_is_a = true;
        g.symmetric = true;
    }
    return oz_gemm(g, s);
}

rt_status rt_debug_chunk_bytes(long long bytes) {
    g_chunk_bytes.store(bytes <= 0 ? kMetricChunkBytes : bytes);
    return RT_OK;
}

rt_status rt_special_dgemm_01(double* ten3_a, int x_a, int y_a, int z_a, int start_x_a, int len_x_a, int start_z_a,
                              int len_z_a, const double* matr_b, int rows_b, int columns_b, int start_row_b,
                              int len_row_b, int start_column_b, int len_column_b, double alpha, double beta,
                              int form, int nslices, void* stream) {
    NvtxRange nvtx_range("rt_special_dgemm_01");
    RT_REQUIRE(x_a >= 0 && y_a >= 0 && z_a >= 0 && rows_b >= 0 && columns_b >= 0,
               "rt_special_dgemm_01: negative dimension");
    RT_REQUIRE(valid_form(form, nslices), "rt_special_dgemm_01: bad form/nslices (%d, %d)", form, nslices);
    RT_REQUIRE(start_x_a >= 0 && len_x_a >= 0 && (int64_t)start_x_a + len_x_a <= x_a && start_z_a >= 0 &&
                   len_z_a >= 0 && (int64_t)start_z_a + len_z_a <= z_a,
               "rt_special_dgemm_01: block of ten3_a outside the tensor");
    RT_REQUIRE(start_row_b >= 0 && len_row_b >= 0 && (int64_t)start_row_b + len_row_b <= rows_b &&
                   start_column_b >= 0 && len_column_b >= 0 && (int64_t)start_column_b + len_column_b <= columns_b,
               "rt_special_dgemm_01: block of matr_b outside the matrix");
    RT_REQUIRE(len_row_b == len_z_a && len_column_b == len_z_a,
               "rt_special_dgemm_01: the block of matr_b must be len_z_a x len_z_a (got %d x %d, len_z_a %d)",
               len_row_b, len_column_b, len_z_a);
    if ((int64_t)len_x_a * y_a * len_z_a == 0) return RT_OK;
    RT_REQUIRE(ten3_a && matr_b, "rt_special_dgemm_01: null pointer");
    return special_dgemm_01(ten3_a, x_a, y_a, start_x_a, len_x_a, start_z_a, len_z_a, matr_b, rows_b, start_row_b,
                            start_column_b, alpha, beta, form, nslices, (cudaStream_t)stream);
}

rt_status rt_ri_ao2mo(const double* C, const double* B, double* ri3mo, int nb, int ns, int naux, int form,
                      int nslices, void* stream) {
    NvtxRange nvtx_range("rt_ri_ao2mo");
    RT_REQUIRE(nb >= 0 && ns >= 0 && naux >= 0, "rt_ri_ao2mo: negative dimension");
    RT_REQUIRE(valid_form(form, nslices), "rt_ri_ao2mo: bad form/nslices (%d, %d)", form, nslices);
    if ((int64_t)nb * ns * naux == 0) return RT_OK;
    RT_REQUIRE(C && B && ri3mo, "rt_ri_ao2mo: null pointer");
    if (form == RT_FORM_FP64) return ri_ao2mo_fp64(C, B, ri3mo, nb, ns, naux, (cudaStream_t)stream);
    return ri_ao2mo_split(C, B, ri3mo, nb, ns, naux, nslices, (cudaStream_t)stream);
}

rt_status rt_ri_ov_k(const double* C, const double* B, int nb, int naux, int nocc, int nvir, double* ov, double* K,
                     int form, int nslices, void* stream) {
    NvtxRange nvtx_range("rt_ri_ov_k");
    RT_REQUIRE(nb >= 0 && naux >= 0 && nocc >= 0 && nvir >= 0, "rt_ri_ov_k: negative dimension");
    RT_REQUIRE(valid_form(form, nslices), "rt_ri_ov_k: bad form/nslices (%d, %d)", form, nslices);
    cudaStream_t s = (cudaStream_t)stream;
    if (K && (nocc == 0 || naux == 0) && nb > 0) RT_CUDA_TRY(cudaMemsetAsync(K, 0, sizeof(double) * nb * (size_t)nb, s));
    if ((int64_t)nb * naux * nocc == 0) {
        if (ov && nocc * (int64_t)nvir * naux > 0)
            RT_CUDA_TRY(cudaMemsetAsync(ov, 0, sizeof(double) * (size_t)nocc * nvir * naux, s));
        return RT_OK;
    }
    RT_REQUIRE(C && B, "rt_ri_ov_k: null input pointer");
    if (form == RT_FORM_FP64) return ri_ov_k_fp64(C, B, nb, naux, nocc, nvir, ov, K, s);
    return ri_ov_k_split(C, B, nb, naux, nocc, nvir, ov, K, nslices, s);
}

// Digit-plane bytes one grouped split launch of the batched entry may hold.
constexpr size_t kBatchPlaneBytes = (size_t)24 << 30;

rt_status rt_ri_ov_k_batched(const rt_ri_problem* probs, int nprob, int form, int nslices, const rt_tuning* tuning,
                             void* stream) {
    NvtxRange nvtx_range("rt_ri_ov_k_batched");
    RT_REQUIRE(nprob >= 0 && (nprob == 0 || probs), "rt_ri_ov_k_batched: bad problem list");
    RT_REQUIRE(valid_form(form, nslices), "rt_ri_ov_k_batched: bad form/nslices (%d, %d)", form, nslices);
    cudaStream_t s = (cudaStream_t)stream;
    size_t xtotal = 0;
    std::vector<size_t> xoff(nprob);
    for (int i = 0; i < nprob; ++i) {
        const rt_ri_problem& q = probs[i];
        RT_REQUIRE(q.nb >= 0 && q.naux >= 0 && q.nocc >= 0 && q.nvir >= 0,
                   "rt_ri_ov_k_batched: problem %d has a negative dimension", i);
        RT_REQUIRE((int64_t)q.nb * q.naux * q.nocc == 0 || (q.C && q.B), "rt_ri_ov_k_batched: problem %d null input", i);
        xoff[i] = xtotal;
        xtotal += (size_t)q.nb * q.nocc * q.naux;
    }
    ScratchBuf xb;
    RT_TRY(scratch_alloc(xb, sizeof(double) * std::max<size_t>(xtotal, 1), s));
    // Problems whose products are empty still get their outputs zeroed.
    for (int i = 0; i < nprob; ++i) {
        const rt_ri_problem& q = probs[i];
        if ((int64_t)q.nocc * q.naux == 0 || q.nb == 0) {
            if (q.K && q.nb) RT_CUDA_TRY(cudaMemsetAsync(q.K, 0, sizeof(double) * q.nb * (size_t)q.nb, s));
            if (q.ov && (int64_t)q.nocc * q.nvir * q.naux > 0)
                RT_CUDA_TRY(cudaMemsetAsync(q.ov, 0, sizeof(double) * (size_t)q.nocc * q.nvir * q.naux, s));
        }
    }
    auto live = [&](const rt_ri_problem& q) { return (int64_t)q.nb * q.naux * q.nocc > 0; };
    double* X = xb.as<double>();
    if (form == RT_FORM_FP64) {
        std::vector<GemmF64> g1, g2, g3;
        for (int i = 0; i < nprob; ++i) {
            const rt_ri_problem& q = probs[i];
            if (!live(q)) continue;
            const int64_t per = (int64_t)q.nb * q.nocc;
            // X = B C_occ as one GEMM over rows (mu, P): A row r at B[r % nb + (r / nb) nb^2],
            // X row r at X[r % nb + (r / nb) nb nocc].
            GemmF64 a;
            a.opa = 'N'; a.opb = 'N'; a.m = (int64_t)q.nb * q.naux; a.n = q.nocc; a.k = q.nb;
            a.A = q.B; a.lda = q.nb; a.a_div = q.nb; a.a_s1 = (int64_t)q.nb * q.nb;
            a.B = q.C; a.ldb = q.nb;
            a.C = X + xoff[i]; a.rsC = 1; a.csC = q.nb; a.c_md = q.nb; a.c_ms1 = per;
            g1.push_back(a);
            if (q.ov && q.nvir > 0) {
                // ov = X^T C_vir over rows (i, P): A row r is X[nb r ..]; ov row r at
                // ov[r % nocc + (r / nocc) nocc nvir].
                GemmF64 b;
                b.opa = 'T'; b.opb = 'N'; b.m = (int64_t)q.nocc * q.naux; b.n = q.nvir; b.k = q.nb;
                b.A = X + xoff[i]; b.lda = q.nb; b.B = q.C + per; b.ldb = q.nb;
                b.C = q.ov; b.rsC = 1; b.csC = q.nocc; b.c_md = q.nocc; b.c_ms1 = (int64_t)q.nocc * q.nvir;
                g2.push_back(b);
            }
            if (q.K) {
                GemmF64 c;
                c.opa = 'N'; c.opb = 'T'; c.m = q.nb; c.n = q.nb; c.k = per / q.nb * q.naux;
                c.A = X + xoff[i]; c.lda = q.nb; c.B = X + xoff[i]; c.ldb = q.nb;
                c.C = q.K; c.rsC = 1; c.csC = q.nb;
                c.splitk = (int)std::max<int64_t>(1, c.k / 4096);  // long contractions: ~4096 terms per item
                g3.push_back(c);
            }
        }
        RT_TRY(gemm_f64_many(g1.data(), (int)g1.size(), s));
        RT_TRY(gemm_f64_many(g2.data(), (int)g2.size(), s));
        RT_TRY(gemm_f64_many(g3.data(), (int)g3.size(), s));
        return RT_OK;
    }
    const int fuse = tuning ? tuning->fuse : 0;
    const int cpi = tuning ? tuning->chunks_per_item : 0;
    std::vector<OzGemm> g1, g2, g3;
    for (int i = 0; i < nprob; ++i) {
        const rt_ri_problem& q = probs[i];
        if (!live(q)) continue;
        const int64_t per = (int64_t)q.nb * q.nocc;
        OzGemm a;
        a.K = q.nb;
        a.A.p = q.B; a.A.rows = (int64_t)q.nb * q.naux; a.A.div = q.nb; a.A.s0 = 1; a.A.s1 = (int64_t)q.nb * q.nb;
        a.A.sk = q.nb;
        a.B.p = q.C; a.B.rows = q.nocc; a.B.s0 = q.nb; a.B.sk = 1;
        a.C.p = X + xoff[i]; a.C.md = q.nb; a.C.ms0 = 1; a.C.ms1 = per; a.C.ns0 = q.nb;
        a.nslices = nslices; a.allow_fuse = fuse != 0; a.chunks_per_item = cpi;
        g1.push_back(a);
        if (q.ov && q.nvir > 0) {
            OzGemm b;
            b.K = q.nb;
            b.A.p = X + xoff[i]; b.A.rows = (int64_t)q.nocc * q.naux; b.A.s0 = q.nb; b.A.sk = 1;
            b.B.p = q.C + per; b.B.rows = q.nvir; b.B.s0 = q.nb; b.B.sk = 1;
            b.C.p = q.ov; b.C.md = q.nocc; b.C.ms0 = 1; b.C.ms1 = (int64_t)q.nocc * q.nvir; b.C.ns0 = q.nocc;
            b.nslices = nslices; b.chunks_per_item = cpi;
            g2.push_back(b);
        }
        if (q.K) {
            OzGemm c;
            c.K = (int64_t)q.nocc * q.naux;
            c.A.p = X + xoff[i]; c.A.rows = q.nb; c.A.s0 = 1; c.A.sk = q.nb;
            c.B = c.A; c.b_is_a = true; c.symmetric = true;
            c.C.p = q.K; c.C.ms0 = 1; c.C.ns0 = q.nb;
            c.nslices = nslices; c.chunks_per_item = cpi;
            g3.push_back(c);
        }
    }
    // Each grouped launch holds the digit planes of all its products at once:
    // flush in sub-batches of at most kBatchPlaneBytes of planes.
    auto run = [&](std::vector<OzGemm>& gs) -> rt_status {
        size_t i0 = 0, bytes = 0;
        for (size_t i = 0; i < gs.size(); ++i) {
            const OzGemm& g = gs[i];
            const size_t b = (size_t)(g.A.rows + (g.b_is_a ? 0 : g.B.rows)) * (size_t)g.K * 2u * (size_t)nslices;
            if (i > i0 && bytes + b > kBatchPlaneBytes) {
                RT_TRY(oz_gemm_many(gs.data() + i0, (int)(i - i0), s));
                i0 = i;
                bytes = 0;
            }
            bytes += b;
        }
        if (i0 < gs.size()) RT_TRY(oz_gemm_many(gs.data() + i0, (int)(gs.size() - i0), s));
        return RT_OK;
    };
    RT_TRY(run(g1));
    RT_TRY(run(g2));
    RT_TRY(run(g3));
    return RT_OK;
}

}  // extern "C"

// ------------------------------------------------ prepared ri3ao (SCF reuse) --

// Digit planes and row exponents of ri3ao as the A operand of the half-transform
// X^P = B^P C_occ, kept on the device that made them.
struct rt_ri3ao_prepared {
    int nb = 0, naux = 0, nslices = 0, device = -1;
    uint16_t* planes = nullptr;
    int* emax = nullptr;
    size_t plane_bytes = 0;
};

extern "C" {

rt_status rt_ri3ao_prepare(const double* B, int nb, int naux, int nslices, rt_ri3ao_prepared** out, void* stream) {
    NvtxRange nvtx_range("rt_ri3ao_prepare");
    RT_REQUIRE(out, "rt_ri3ao_prepare: null handle pointer");
    *out = nullptr;
    RT_REQUIRE(nb > 0 && naux > 0, "rt_ri3ao_prepare: nb and naux must be positive");
    RT_REQUIRE(nslices >= 3 && nslices <= 8, "rt_ri3ao_prepare: nslices must be in 3..8");
    RT_REQUIRE(B, "rt_ri3ao_prepare: null ri3ao");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t rows = (int64_t)nb * naux;
    auto* h = new rt_ri3ao_prepared;
    h->nb = nb; h->naux = naux; h->nslices = nslices;
    h->plane_bytes = oz_plane_bytes(rows, nb, nslices);
    auto fail = [&](rt_status st) {
        if (h->planes) cudaFree(h->planes);
        if (h->emax) cudaFree(h->emax);
        delete h;
        return st;
    };
    cudaError_t e = cudaGetDevice(&h->device);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->planes, h->plane_bytes);
    if (e == cudaSuccess) e = cudaMalloc((void**)&h->emax, sizeof(int) * (size_t)rows);
    if (e != cudaSuccess) {
        cudaGetLastError();
        const rt_status st = e == cudaErrorMemoryAllocation ? RT_ERR_NO_MEMORY : RT_ERR_CUDA;
        set_error(st, "rt_ri3ao_prepare: %zu bytes of digit planes: %s", h->plane_bytes, cudaGetErrorString(e));
        return fail(st);
    }
    rt_status st = error_word_reset(s);
    if (st != RT_OK) return fail(st);
    OzOperand A;  // rows (mu, P), k = nu: B[mu + nb nu + nb^2 P], as in x_product
    A.p = B; A.rows = rows; A.div = nb; A.s0 = 1; A.s1 = (int64_t)nb * nb; A.sk = nb;
    st = oz_slice_into(A, nb, nslices, h->planes, h->emax, s);
    if (st == RT_OK) st = error_word_check(s, "rt_ri3ao_prepare");  // synchronises: the handle is ready
    if (st != RT_OK) return fail(st);
    *out = h;
    return RT_OK;
}

rt_status rt_ri3ao_prepared_bytes(const rt_ri3ao_prepared* h, long long* bytes) {
    RT_REQUIRE(h && bytes, "rt_ri3ao_prepared_bytes: null argument");
    *bytes = (long long)(h->plane_bytes + sizeof(int) * (size_t)h->nb * h->naux);
    return RT_OK;
}

rt_status rt_ri_ov_k_prepared(const rt_ri3ao_prepared* h, const double* C, int nocc, int nvir, double* ov, double* K,
                              void* stream) {
    NvtxRange nvtx_range("rt_ri_ov_k_prepared");
    RT_REQUIRE(h, "rt_ri_ov_k_prepared: null handle");
    RT_REQUIRE(nocc >= 0 && nvir >= 0, "rt_ri_ov_k_prepared: negative dimension");
    int dev = -1;
    RT_CUDA_TRY(cudaGetDevice(&dev));
    RT_REQUIRE(dev == h->device, "rt_ri_ov_k_prepared: handle made on device %d, current device %d", h->device, dev);
    cudaStream_t s = (cudaStream_t)stream;
    const int nb = h->nb, naux = h->naux, S = h->nslices;
    if (K && nocc == 0) RT_CUDA_TRY(cudaMemsetAsync(K, 0, sizeof(double) * nb * (size_t)nb, s));
    if (nocc == 0) return RT_OK;
    RT_REQUIRE(C, "rt_ri_ov_k_prepared: null C");
    const int64_t per = (int64_t)nb * nocc;
    ScratchBuf xb;
    RT_TRY(scratch_alloc(xb, sizeof(double) * (size_t)(per * naux), s));
    double* X = xb.as<double>();
    OzGemm g = x_product(C, nullptr, nb, naux, nocc, X, S);
    g.a_planes = h->planes;
    g.a_emax = h->emax;
    RT_TRY(oz_gemm(g, s));
    if (ov && nvir > 0) RT_TRY(oz_gemm(ov_product(C, nb, naux, nocc, nvir, X, ov, S), s));
    if (K) RT_TRY(ri_k_from_x(X, nb, nocc, naux, K, RT_FORM_SPLIT, S, s));
    return RT_OK;
}

rt_status rt_ri3ao_release(rt_ri3ao_prepared* h) {
    if (!h) return RT_OK;
    int cur = -1;
    cudaGetDevice(&cur);
    if (cur != h->device) cudaSetDevice(h->device);
    cudaFree(h->planes);
    cudaFree(h->emax);
    if (cur != h->device && cur >= 0) cudaSetDevice(cur);
    delete h;
    return RT_OK;
}

rt_status rt_ri_j(const double* B, const double* D, int nb, int naux, double* w, double* J, void* stream) {
    NvtxRange nvtx_range("rt_ri_j");
    RT_REQUIRE(nb >= 0 && naux >= 0, "rt_ri_j: negative dimension");
    cudaStream_t s = (cudaStream_t)stream;
    if (naux == 0) {
        if (J && nb) RT_CUDA_TRY(cudaMemsetAsync(J, 0, sizeof(double) * nb * (size_t)nb, s));
        return RT_OK;
    }
    if (nb == 0) {
        if (w) RT_CUDA_TRY(cudaMemsetAsync(w, 0, sizeof(double) * naux, s));
        return RT_OK;
    }
    RT_REQUIRE(B && D, "rt_ri_j: null input pointer");
    return ri_j_fp64(B, D, nb, naux, w, J, s);
}

rt_status rt_ri_j_symmetric(const double* B, const double* D, int nb, int naux, double* w, double* J, void* stream) {
    NvtxRange nvtx_range("rt_ri_j_symmetric");
    RT_REQUIRE(nb >= 0 && naux >= 0, "rt_ri_j_symmetric: negative dimension");
    cudaStream_t s = (cudaStream_t)stream;
    if (naux == 0) {
        if (J && nb) RT_CUDA_TRY(cudaMemsetAsync(J, 0, sizeof(double) * nb * (size_t)nb, s));
        return RT_OK;
    }
    if (nb == 0) {
        if (w) RT_CUDA_TRY(cudaMemsetAsync(w, 0, sizeof(double) * naux, s));
        return RT_OK;
    }
    RT_REQUIRE(B && D, "rt_ri_j_symmetric: null input pointer");
    if (symmetry_check_enabled()) {
        RT_TRY(symmetry_sample(B, nb, naux, s));
        RT_TRY(symmetry_sample(D, nb, 1, s));
    }
    return ri_j_fp64_symmetric(B, D, nb, naux, w, J, s);
}

rt_status rt_ri_exchange_energy(const double* D, const double* K, int nb, double* ex_device, void* stream) {
    NvtxRange nvtx_range("rt_ri_exchange_energy");
    RT_REQUIRE(nb >= 0 && ex_device, "rt_ri_exchange_energy: bad argument");
    return exchange_energy(D, K, nb, ex_device, (cudaStream_t)stream);
}

rt_status rt_synth_ri3ao(uint64_t seed, int nb, int P0, int nslab, double* B, void* stream) {
    RT_REQUIRE(nb >= 0 && P0 >= 0 && nslab >= 0, "rt_synth_ri3ao: negative argument");
    return synth_ri3ao(seed, nb, P0, nslab, B, (cudaStream_t)stream);
}

rt_status rt_synth_delta(uint64_t seed, long long nov, double* d, void* stream) {
    RT_REQUIRE(nov >= 0 && (nov == 0 || d), "rt_synth_delta: bad arguments");
    return synth_delta(seed, nov, d, (cudaStream_t)stream);
}

rt_status rt_synth_coef_seed(uint64_t seed, int nb, double* M, void* stream) {
    RT_REQUIRE(nb >= 0, "rt_synth_coef_seed: negative size");
    return synth_coef_seed(seed, nb, M, (cudaStream_t)stream);
}

}  // extern "C"

namespace rt {
namespace {

// Strict lower triangle of every [nb x nb] slab from its upper triangle:
// block (tx, ty) of CTA (P, I >= J) reads the 32 x 32 tile of rows J, columns I
// and writes its transpose to rows I, columns J through shared memory (in a
// diagonal tile, only the elements below the diagonal).
__global__ void __launch_bounds__(256) sym_mirror_kernel(double* __restrict__ B, int nb, int nbt, int64_t np) {
    __shared__ double t[32][33];
    const int64_t pairs = (int64_t)nbt * (nbt + 1) / 2;  // tiles on or below the diagonal
    const int64_t idx = blockIdx.x;
    const int64_t P = idx / pairs;
    if (P >= np) return;
    int64_t q = idx % pairs;
    int I = 0;
    while (q >= I + 1) {  // row-major enumeration of (I, J), J <= I
        q -= I + 1;
        ++I;
    }
    const int J = (int)q;
    double* slab = B + P * (int64_t)nb * nb;
    const int tx = threadIdx.x, ty = threadIdx.y;
    // upper tile: rows mu = J*32 + tx, columns nu = I*32 + r  (mu < nu)
    for (int r = ty; r < 32; r += 8) {
        const int mu = J * 32 + tx, nu = I * 32 + r;
        if (mu < nb && nu < nb) t[r][tx] = slab[mu + (int64_t)nb * nu];
    }
    __syncthreads();
    // lower tile: rows nu = I*32 + tx, columns mu = J*32 + r
    for (int r = ty; r < 32; r += 8) {
        const int nu = I * 32 + tx, mu = J * 32 + r;
        if (mu < nb && nu < nb && nu > mu) slab[nu + (int64_t)nb * mu] = t[tx][r];
    }
}

// Zero-copy form for page-locked host memory: a small grid reads the upper
// 32x32 tiles (I <= J; in a diagonal tile the upper half) of every slab straight
// from host memory over the host link and writes each tile and its mirror to
// device memory.  Few CTAs suffice to keep the link busy, so most SMs stay free
// for the transform of the previous slab block.
__global__ void __launch_bounds__(256) sym_gather_kernel(const double* __restrict__ hB, double* __restrict__ dB,
                                                         int nb, int nbt, int64_t np) {
    __shared__ double t[32][33];
    const int64_t pairs = (int64_t)nbt * (nbt + 1) / 2;
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int64_t idx = blockIdx.x; idx < np * pairs; idx += gridDim.x) {
        const int64_t P = idx / pairs;
        int64_t q = idx % pairs;
        int J = 0;
        while (q >= J + 1) {  // column-block-major enumeration of (I, J), I <= J
            q -= J + 1;
            ++J;
        }
        const int I = (int)q;
        const double* src = hB + P * (int64_t)nb * nb;
        double* dst = dB + P * (int64_t)nb * nb;
        // upper tile: rows mu = I*32 + tx, columns nu = J*32 + r
        for (int r = ty; r < 32; r += 8) {
            const int mu = I * 32 + tx, nu = J * 32 + r;
            if (mu < nb && nu < nb && mu <= nu) {
                const double v = src[mu + (int64_t)nb * nu];
                t[r][tx] = v;
                dst[mu + (int64_t)nb * nu] = v;
            }
        }
        __syncthreads();
        // mirror: rows nu = J*32 + tx, columns mu = I*32 + r, below the diagonal
        for (int r = ty; r < 32; r += 8) {
            const int nu = J * 32 + tx, mu = I * 32 + r;
            if (mu < nb && nu < nb && nu > mu) dst[nu + (int64_t)nb * mu] = t[tx][r];
        }
        __syncthreads();
    }
}

// dst[0, n) = src[0, n) where src is the device view of page-locked host
// memory: the SMs read the host pages directly, four 16-byte loads in flight
// per thread.  Used for whole ri3ao slabs when they are pinned.
__global__ void __launch_bounds__(256) host_read_kernel(const double2* __restrict__ src, double2* __restrict__ dst,
                                                        int64_t n2) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (; i + 3 * stride < n2; i += 4 * stride) {
        const double2 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
        dst[i] = a;
        dst[i + stride] = b;
        dst[i + 2 * stride] = c;
        dst[i + 3 * stride] = d;
    }
    for (; i < n2; i += stride) dst[i] = src[i];
}

// Device view of the page-locked host range h[0, n), or nullptr when the range
// is not page-locked as a whole: its first and its last element must both be
// pinned, with device addresses n - 1 elements apart (one registration, or
// registrations mapped contiguously).  Anything else (pageable memory, a range
// only partly registered) goes through the copy engine.
const double* pinned_view(const double* h, int64_t n) {
    if (n <= 0) return nullptr;
    cudaPointerAttributes a{}, b{};
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess || a.type != cudaMemoryTypeHost || !a.devicePointer ||
        cudaPointerGetAttributes(&b, h + (n - 1)) != cudaSuccess || b.type != cudaMemoryTypeHost ||
        !b.devicePointer ||
        (const double*)b.devicePointer != (const double*)a.devicePointer + (n - 1)) {
        cudaGetLastError();  // pageable memory has no device view
        return nullptr;
    }
    return static_cast<const double*>(a.devicePointer);
}

// Host-to-device copy of n doubles: the kernel above for 16-byte-aligned
// pinned memory, the copy engine otherwise.
rt_status copy_slabs_h2d(const double* hB, double* dB, int64_t n, cudaStream_t s) {
    const double* view = ((n & 1) == 0 && ((uintptr_t)hB & 15) == 0 && ((uintptr_t)dB & 15) == 0)
                             ? pinned_view(hB, n) : nullptr;
    if (view && ((uintptr_t)view & 15) == 0) {
        host_read_kernel<<<2 * sm_count(), 256, 0, s>>>(reinterpret_cast<const double2*>(view),
                                                         reinterpret_cast<double2*>(dB), n / 2);
        return check_launch("host_read_kernel");
    }
    RT_CUDA_TRY(cudaMemcpyAsync(dB, hB, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, s));
    return RT_OK;
}

// Host-to-device copy of slabs P0 .. P0+np-1 of a symmetric ri3ao reading only
// (about) the upper triangle: for each 32-column block J, rows 0 .. 32J+31 of
// those columns of every slab form one 3-D box (row pitch nb, slab pitch nb^2).
// Everything below the diagonal is then mirrored on the device.
rt_status copy_symmetric_slabs(const double* hB, double* dB, int nb, int64_t np, cudaStream_t s) {
    const int nbt = (nb + 31) / 32;
    if (const double* dev_view = pinned_view(hB, (int64_t)nb * nb * np)) {
        // Two CTAs per SM keep enough host reads in flight to fill the link (1, 0.5 and
        // 0.1 per SM left it idle; 4 and 8 per SM took SMs from the transform).
        sym_gather_kernel<<<2 * sm_count(), dim3(32, 8), 0, s>>>(dev_view, dB, nb, nbt, np);
        return check_launch("sym_gather_kernel");
    }
    for (int J = 0; J < nbt; ++J) {
        const int c0 = 32 * J, c1 = std::min(nb, c0 + 32);
        const int rows = std::min(nb, c0 + 32);
        cudaMemcpy3DParms m = {};
        m.srcPtr = make_cudaPitchedPtr(const_cast<double*>(hB) + (size_t)nb * c0, sizeof(double) * nb,
                                       sizeof(double) * nb, nb);
        m.dstPtr = make_cudaPitchedPtr(dB + (size_t)nb * c0, sizeof(double) * nb, sizeof(double) * nb, nb);
        m.extent = make_cudaExtent(sizeof(double) * rows, (size_t)(c1 - c0), (size_t)np);
        m.kind = cudaMemcpyHostToDevice;
        RT_CUDA_TRY(cudaMemcpy3DAsync(&m, s));
    }
    const int64_t blocks = np * ((int64_t)nbt * (nbt + 1) / 2);
    sym_mirror_kernel<<<(unsigned)blocks, dim3(32, 8), 0, s>>>(dB, nb, nbt, np);
    return check_launch("sym_mirror_kernel");
}

// The pipelined host-pointer entry; symmetric: ri3ao slabs are symmetric and
// only their upper triangles cross the host link.
rt_status ri_ov_k_host_impl(const double* C, const double* B, int nb, int naux, int nocc, int nvir, double* ov,
                            double* K, int form, int nslices, void* stream, bool symmetric) {
    RT_REQUIRE(nb >= 0 && naux >= 0 && nocc >= 0 && nvir >= 0, "rt_ri_ov_k_host: negative dimension");
    RT_REQUIRE(valid_form(form, nslices), "rt_ri_ov_k_host: bad form/nslices");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nC = (size_t)nb * (nocc + nvir), nB = (size_t)nb * nb * naux;
    const size_t nO = (size_t)nocc * nvir * naux, nK = (size_t)nb * nb;
    const int64_t per = (int64_t)nb * nocc, slab = (int64_t)nb * nb, oslab = (int64_t)nocc * nvir;
    if (nB == 0 || nocc == 0) {
        if (ov && nO) memset(ov, 0, sizeof(double) * nO);
        if (K && nK) memset(K, 0, sizeof(double) * nK);
        return RT_OK;
    }
    ScratchBuf dC, dB, dX, dO, dK;
    RT_TRY(scratch_alloc(dC, sizeof(double) * nC, s));
    RT_TRY(scratch_alloc(dB, sizeof(double) * nB, s));
    RT_TRY(scratch_alloc(dX, sizeof(double) * (size_t)per * naux, s));
    if (ov && nO) RT_TRY(scratch_alloc(dO, sizeof(double) * nO, s));
    if (K) RT_TRY(scratch_alloc(dK, sizeof(double) * nK, s));
    RT_TRY(error_word_reset(s));

    // Slab blocks of ~512 MB: host-to-device copies of block b+1 run on their own
    // stream while block b is transformed; ov blocks go back on a third stream.
    const int64_t blk = std::max<int64_t>(1, std::min<int64_t>(naux, ((int64_t)64 << 20) / std::max<int64_t>(slab, 1)));
    // Block boundaries: full blocks, then a short last block (a sixth of one), so
    // that little transform work is left once the last slabs have arrived.
    std::vector<int64_t> bstart;
    {
        const int64_t tail = naux > blk ? std::max<int64_t>(1, blk / 6) : naux;
        for (int64_t P = 0; P < naux - tail; P += blk) bstart.push_back(P);
        bstart.push_back(naux - tail);
        bstart.push_back(naux);
    }
    const int64_t nblk = (int64_t)bstart.size() - 1;
    cudaStream_t hs = nullptr, ds = nullptr;
    cudaEvent_t ready = nullptr;
    std::vector<cudaEvent_t> in(nblk, nullptr), out(nblk, nullptr);
    rt_status st = RT_OK;
    auto fail = [&](cudaError_t e, const char* what) {
        set_error(RT_ERR_CUDA, "rt_ri_ov_k_host: %s: %s", what, cudaGetErrorString(e));
        st = RT_ERR_CUDA;
    };
    cudaError_t e;
    {
        int lo = 0, hi = 0;  // the copy stream gets the highest priority: its CTAs go first
        cudaDeviceGetStreamPriorityRange(&lo, &hi);
        if ((e = cudaStreamCreateWithPriority(&hs, cudaStreamNonBlocking, hi)) != cudaSuccess) fail(e, "stream");
    }
    if (st == RT_OK && (e = cudaStreamCreateWithFlags(&ds, cudaStreamNonBlocking)) != cudaSuccess) fail(e, "stream");
    if (st == RT_OK && (e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming)) != cudaSuccess) fail(e, "event");
    for (int64_t b = 0; st == RT_OK && b < nblk; ++b) {
        if ((e = cudaEventCreateWithFlags(&in[b], cudaEventDisableTiming)) != cudaSuccess) fail(e, "event");
        else if ((e = cudaEventCreateWithFlags(&out[b], cudaEventDisableTiming)) != cudaSuccess) fail(e, "event");
    }
    if (st == RT_OK && (e = cudaMemcpyAsync(dC.p, C, sizeof(double) * nC, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        fail(e, "host-to-device copy");
    if (st == RT_OK) {
        // The pool allocations above are ordered on `s`; the copy streams start after them.
        cudaEventRecord(ready, s);
        cudaStreamWaitEvent(hs, ready, 0);
        cudaStreamWaitEvent(ds, ready, 0);
        auto compute = [&](int64_t b) -> rt_status {
            const int64_t P0 = bstart[b], np = bstart[b + 1] - bstart[b];
            cudaStreamWaitEvent(s, in[b], 0);
            RT_TRY(ri_ov_block(dC.as<double>(), dB.as<double>() + P0 * slab, nb, np, nocc, nvir,
                               dX.as<double>() + P0 * per, (ov && nO) ? dO.as<double>() + P0 * oslab : nullptr, form,
                               nslices, s));
            if (ov && nO) {
                cudaEventRecord(out[b], s);
                cudaStreamWaitEvent(ds, out[b], 0);
                RT_CUDA_TRY(cudaMemcpyAsync(ov + P0 * oslab, dO.as<double>() + P0 * oslab,
                                            sizeof(double) * (size_t)(np * oslab), cudaMemcpyDeviceToHost, ds));
            }
            return RT_OK;
        };
        for (int64_t b = 0; st == RT_OK && b < nblk; ++b) {
            const int64_t P0 = bstart[b], np = bstart[b + 1] - bstart[b];
            if (symmetric) {
                st = copy_symmetric_slabs(B + P0 * slab, dB.as<double>() + P0 * slab, nb, np, hs);
                if (st != RT_OK) break;
            } else {
                st = copy_slabs_h2d(B + P0 * slab, dB.as<double>() + P0 * slab, np * slab, hs);
                if (st != RT_OK) break;
            }
            cudaEventRecord(in[b], hs);
            if (b > 0) st = compute(b - 1);
        }
        if (st == RT_OK) st = compute(nblk - 1);
        if (st == RT_OK && K) {
            st = ri_k_from_x(dX.as<double>(), nb, nocc, naux, dK.as<double>(), form, nslices, s);
            if (st == RT_OK && (e = cudaMemcpyAsync(K, dK.p, sizeof(double) * nK, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
                fail(e, "device-to-host copy");
        }
    }
    // Drain both copy streams before the scratch is released on `s`.
    if (hs) cudaStreamSynchronize(hs);
    if (ds) cudaStreamSynchronize(ds);
    cudaStreamSynchronize(s);
    for (auto ev : in) if (ev) cudaEventDestroy(ev);
    for (auto ev : out) if (ev) cudaEventDestroy(ev);
    if (ready) cudaEventDestroy(ready);
    if (hs) cudaStreamDestroy(hs);
    if (ds) cudaStreamDestroy(ds);
    if (st != RT_OK) return st;
    return error_word_check(s, "rt_ri_ov_k_host");
}

// Host-buffer full transform, pipelined over the host link.
//   Phase 1, per slab block b: ri3ao slabs of block b arrive on the copy stream
//   while the half-transform T^P = B^P C of block b-1 runs.
//   Phase 2, per block of q columns: ri3mo[:, :, q0:q1] = sum_mu C[mu,p] T^P[mu,q]
//   for every P is contiguous in the P-fastest layout, so its copy to the host
//   overlaps the next column block's GEMM.  ri3mo reuses ri3ao's device buffer
//   (phase 2 starts after every read of B on the same stream).
// Every output element is computed exactly as by rt_ri_ao2mo: the column
// blocks change which rows share a launch, not what any element sums.
rt_status ri_ao2mo_host_impl(const double* C, const double* B, double* R, int nb, int ns, int naux, int form,
                             int nslices, cudaStream_t s) {
    RT_REQUIRE(nb >= 0 && ns >= 0 && naux >= 0, "ri_ao2mo host: negative dimension");
    RT_REQUIRE(valid_form(form, nslices), "ri_ao2mo host: bad form/nslices (%d, %d)", form, nslices);
    const size_t nR = (size_t)naux * ns * ns;
    if (nR == 0) return RT_OK;
    if (nb == 0) {
        memset(R, 0, sizeof(double) * nR);
        return RT_OK;
    }
    RT_REQUIRE(C && B && R, "ri_ao2mo host: null pointer");
    const int64_t slab = (int64_t)nb * nb, per = (int64_t)nb * ns;
    const size_t nB = (size_t)slab * naux;
    ScratchBuf dC, dB, dT, dRx;
    RT_TRY(scratch_alloc(dC, sizeof(double) * (size_t)per, s));
    RT_TRY(scratch_alloc(dB, sizeof(double) * nB, s));
    RT_TRY(scratch_alloc(dT, sizeof(double) * (size_t)per * naux, s));
    double* dR = dB.as<double>();
    if (nR > nB) {
        RT_TRY(scratch_alloc(dRx, sizeof(double) * nR, s));
        dR = dRx.as<double>();
    }
    RT_TRY(error_word_reset(s));
    // ~512 MB per slab block and per ri3mo column block.
    const int64_t sblk = std::max<int64_t>(1, std::min<int64_t>(naux, ((int64_t)64 << 20) / std::max<int64_t>(slab, 1)));
    const int64_t qcol = (int64_t)naux * ns;  // elements of one ri3mo column q
    const int64_t qblk = std::max<int64_t>(1, std::min<int64_t>(ns, ((int64_t)64 << 20) / std::max<int64_t>(qcol, 1)));
    const int64_t nsb = ceil_div(naux, sblk), nqb = ceil_div(ns, qblk);
    cudaStream_t hs = nullptr, ds = nullptr;
    cudaEvent_t ready = nullptr;
    std::vector<cudaEvent_t> in(nsb, nullptr), out(nqb, nullptr);
    rt_status st = RT_OK;
    auto fail = [&](cudaError_t e, const char* what) {
        set_error(RT_ERR_CUDA, "ri_ao2mo host: %s: %s", what, cudaGetErrorString(e));
        st = RT_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&hs, cudaStreamNonBlocking)) != cudaSuccess) fail(e, "stream");
    if (st == RT_OK && (e = cudaStreamCreateWithFlags(&ds, cudaStreamNonBlocking)) != cudaSuccess) fail(e, "stream");
    if (st == RT_OK && (e = cudaEventCreateWithFlags(&ready, cudaEventDisableTiming)) != cudaSuccess) fail(e, "event");
    for (int64_t b = 0; st == RT_OK && b < nsb; ++b)
        if ((e = cudaEventCreateWithFlags(&in[b], cudaEventDisableTiming)) != cudaSuccess) fail(e, "event");
    for (int64_t j = 0; st == RT_OK && j < nqb; ++j)
        if ((e = cudaEventCreateWithFlags(&out[j], cudaEventDisableTiming)) != cudaSuccess) fail(e, "event");
    if (st == RT_OK && (e = cudaMemcpyAsync(dC.p, C, sizeof(double) * (size_t)per, cudaMemcpyHostToDevice, s)) !=
                           cudaSuccess)
        fail(e, "host-to-device copy");
    if (st == RT_OK) {
        // The pool allocations above are ordered on `s`; the copy streams start after them.
        cudaEventRecord(ready, s);
        cudaStreamWaitEvent(hs, ready, 0);
        cudaStreamWaitEvent(ds, ready, 0);
        const double* Cd = dC.as<double>();
        auto half = [&](int64_t b) -> rt_status {
            const int64_t P0 = b * sblk, np = std::min<int64_t>(sblk, naux - P0);
            cudaStreamWaitEvent(s, in[b], 0);
            const double* Bb = dB.as<double>() + P0 * slab;
            double* Tb = dT.as<double>() + P0 * per;
            if (form == RT_FORM_FP64) {
                GemmF64 g1;
                g1.opa = 'N'; g1.opb = 'N'; g1.m = nb; g1.n = ns; g1.k = nb;
                g1.A = Bb; g1.lda = nb; g1.sA = slab;
                g1.B = Cd; g1.ldb = nb; g1.sB = 0;
                g1.C = Tb; g1.rsC = 1; g1.csC = nb; g1.bsC = per; g1.batch = np;
                return gemm_f64(g1, s);
            }
            return oz_gemm(t_product(Cd, Bb, nb, ns, np, Tb, nslices), s);
        };
        for (int64_t b = 0; st == RT_OK && b < nsb; ++b) {
            const int64_t P0 = b * sblk, np = std::min<int64_t>(sblk, naux - P0);
            st = copy_slabs_h2d(B + P0 * slab, dB.as<double>() + P0 * slab, np * slab, hs);
            if (st != RT_OK) break;
            cudaEventRecord(in[b], hs);
            if (b > 0) st = half(b - 1);
        }
        if (st == RT_OK) st = half(nsb - 1);
        auto second = [&](int64_t j) -> rt_status {
            const int64_t q0 = j * qblk, nq = std::min<int64_t>(qblk, ns - q0);
            double* Rq = dR + qcol * q0;
            const double* Tq = dT.as<double>() + (int64_t)nb * q0;
            if (form == RT_FORM_FP64) {
                GemmF64 g2;
                g2.opa = 'T'; g2.opb = 'N'; g2.m = ns; g2.n = nq; g2.k = nb;
                g2.A = Cd; g2.lda = nb; g2.sA = 0;
                g2.B = Tq; g2.ldb = nb; g2.sB = per;
                g2.C = Rq; g2.rsC = naux; g2.csC = qcol; g2.bsC = 1; g2.batch = naux;
                return gemm_f64(g2, s);
            }
            return oz_gemm(r_product(Cd, Tq, nb, ns, nq, naux, naux, Rq, nslices), s);
        };
        // Each column block's copy is queued after the next block's GEMM, so a copy to
        // pageable memory (which returns only when done) still overlaps device work.
        for (int64_t j = 0; st == RT_OK && j <= nqb; ++j) {
            if (j < nqb) {
                st = second(j);
                if (st != RT_OK) break;
                cudaEventRecord(out[j], s);
            }
            if (j > 0) {
                const int64_t q0 = (j - 1) * qblk, nq = std::min<int64_t>(qblk, ns - q0);
                cudaStreamWaitEvent(ds, out[j - 1], 0);
                if ((e = cudaMemcpyAsync(R + qcol * q0, dR + qcol * q0, sizeof(double) * (size_t)(qcol * nq),
                                         cudaMemcpyDeviceToHost, ds)) != cudaSuccess)
                    fail(e, "device-to-host copy");
            }
        }
    }
    if (hs) cudaStreamSynchronize(hs);
    if (ds) cudaStreamSynchronize(ds);
    cudaStreamSynchronize(s);
    for (auto ev : in) if (ev) cudaEventDestroy(ev);
    for (auto ev : out) if (ev) cudaEventDestroy(ev);
    if (ready) cudaEventDestroy(ready);
    if (hs) cudaStreamDestroy(hs);
    if (ds) cudaStreamDestroy(ds);
    if (st != RT_OK) return st;
    return error_word_check(s, "ri_ao2mo host");
}

// Precision form of the Fortran-ABI drop-ins, read once per process from the
// environment: RT_FORM = fp64 (default) | split, RT_NSLICES = 3..8 (default 7).
// Unchanged callers therefore keep float64 parity; a deployment opts in to the
// split form without relinking.  An unrecognised value makes every drop-in call
// fail (rt_last_status) rather than silently run another form.
struct SeamForm {
    int form = RT_FORM_FP64;
    int nslices = 7;
    bool ok = true;
    char why[160] = {0};
};

const SeamForm& seam_form() {
    static const SeamForm f = [] {
        SeamForm r;
        if (const char* v = getenv("RT_FORM")) {
            if (!strcasecmp(v, "split")) r.form = RT_FORM_SPLIT;
            else if (strcasecmp(v, "fp64") && *v) {
                r.ok = false;
                snprintf(r.why, sizeof(r.why), "RT_FORM=%s: expected fp64 or split", v);
            }
        }
        if (const char* v = getenv("RT_NSLICES")) {
            char* end = nullptr;
            const long n = strtol(v, &end, 10);
            if (*v && end && *end == 0 && n >= 3 && n <= 8) r.nslices = (int)n;
            else if (*v) {
                r.ok = false;
                snprintf(r.why, sizeof(r.why), "RT_NSLICES=%s: expected an integer in 3..8", v);
            }
        }
        return r;
    }();
    return f;
}

rt_status seam_check(const char* who) {
    const SeamForm& f = seam_form();
    if (!f.ok) {
        set_error(RT_ERR_INVALID_ARG, "%s: %s", who, f.why);
        return RT_ERR_INVALID_ARG;
    }
    return RT_OK;
}

// C block <- alpha * P + beta * C block (column-major, leading dimension ldc;
// beta == 0 does not read C).
__global__ void __launch_bounds__(256) axpby_block_kernel(double* __restrict__ Cb, int64_t ldc,
                                                          const double* __restrict__ P, int64_t m, int64_t n,
                                                          double alpha, double beta) {
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < m * n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % m, j = idx / m;
        double* c = Cb + i + j * ldc;
        *c = beta == 0.0 ? alpha * P[idx] : fma(beta, *c, alpha * P[idx]);
    }
}

}  // namespace
}  // namespace rt

extern "C" {

rt_status rt_ri_ao2mo_host(const double* C, const double* B, double* ri3mo, int nb, int ns, int naux, int form,
                           int nslices, void* stream) {
    NvtxRange nvtx_range("rt_ri_ao2mo_host");
    return ri_ao2mo_host_impl(C, B, ri3mo, nb, ns, naux, form, nslices, (cudaStream_t)stream);
}

rt_status rt_ri_ov_k_host(const double* C, const double* B, int nb, int naux, int nocc, int nvir, double* ov,
                          double* K, int form, int nslices, void* stream) {
    NvtxRange nvtx_range("rt_ri_ov_k_host");
    return ri_ov_k_host_impl(C, B, nb, naux, nocc, nvir, ov, K, form, nslices, stream, false);
}

rt_status rt_ri_ov_k_host_symmetric(const double* C, const double* B, int nb, int naux, int nocc, int nvir,
                                    double* ov, double* K, int form, int nslices, void* stream) {
    NvtxRange nvtx_range("rt_ri_ov_k_host_symmetric");
    if (symmetry_check_enabled() && B && nb > 0)
        RT_TRY(symmetry_sample_host(B, nb, naux, "rt_ri_ov_k_host_symmetric"));
    return ri_ov_k_host_impl(C, B, nb, naux, nocc, nvir, ov, K, form, nslices, stream, true);
}

// ------------------------------------------------------------ Fortran seam --

void ri_ao2mo_f_(const double* eigenvector, const double* ri3fn, double* ri3mo, const int* num_states,
                 const int* num_basis, const int* num_auxbas) {
    NvtxRange nvtx_range("ri_ao2mo_f_");
    rt::set_error(RT_OK, "");
    const int ns = *num_states, nb = *num_basis, naux = *num_auxbas;
    const size_t nR = (ns > 0 && naux > 0) ? (size_t)naux * ns * ns : 0;
    auto run = [&]() -> rt_status {
        RT_TRY(seam_check("ri_ao2mo_f_"));
        if (nR == 0) return RT_OK;
        if (nb <= 0) {
            memset(ri3mo, 0, sizeof(double) * nR);
            return RT_OK;
        }
        const SeamForm& f = seam_form();
        return ri_ao2mo_host_impl(eigenvector, ri3fn, ri3mo, nb, ns, naux, f.form, f.nslices, cudaStreamPerThread);
    };
    if (run() != RT_OK) {
        // The Fortran zero-fills ri3mo first (restmatr.f90:178): a failed call leaves that state.
        if (nR) memset(ri3mo, 0, sizeof(double) * nR);
        fprintf(stderr, "ri_ao2mo_f_: %s\n", rt_last_error());
    }
}

void general_dgemm_f_(const double* matr_a, const int* rows_a, const int* columns_a, const int* start_row_a,
                      const int* len_row_a, const int* start_column_a, const int* len_column_a, const char* opa,
                      const double* matr_b, const int* rows_b, const int* columns_b, const int* start_row_b,
                      const int* len_row_b, const int* start_column_b, const int* len_column_b, const char* opb,
                      double* matr_c, const int* rows_c, const int* columns_c, const int* start_row_c,
                      const int* len_row_c, const int* start_column_c, const int* len_column_c,
                      const double* alpha, const double* beta) {
    NvtxRange nvtx_range("general_dgemm_f_");
    rt::set_error(RT_OK, "");
    auto run = [&]() -> rt_status {
        const char oa = *opa, ob = *opb;
        RT_REQUIRE(oa == 'N' || oa == 'T', "general_dgemm_f_: opa must be 'N' or 'T'");
        RT_REQUIRE(ob == 'N' || ob == 'T', "general_dgemm_f_: opb must be 'N' or 'T'");
        const int m = *len_row_c, n = *len_column_c;
        const int k = oa == 'N' ? *len_column_a : *len_row_a;
        const int am = oa == 'N' ? *len_row_a : *len_column_a;
        const int bk = ob == 'N' ? *len_row_b : *len_column_b;
        const int bn = ob == 'N' ? *len_column_b : *len_row_b;
        RT_REQUIRE(am == m && bk == k && bn == n, "general_dgemm_f_: inconsistent block shapes");
        RT_REQUIRE(*start_row_a >= 0 && *start_row_a + *len_row_a <= *rows_a && *start_column_a >= 0 &&
                       *start_column_a + *len_column_a <= *columns_a,
                   "general_dgemm_f_: block of A outside the matrix");
        RT_REQUIRE(*start_row_b >= 0 && *start_row_b + *len_row_b <= *rows_b && *start_column_b >= 0 &&
                       *start_column_b + *len_column_b <= *columns_b,
                   "general_dgemm_f_: block of B outside the matrix");
        RT_REQUIRE(*start_row_c >= 0 && *start_row_c + m <= *rows_c && *start_column_c >= 0 &&
                       *start_column_c + n <= *columns_c,
                   "general_dgemm_f_: block of C outside the matrix");
        RT_TRY(seam_check("general_dgemm_f_"));
        if (m == 0 || n == 0) return RT_OK;
        cudaStream_t s = cudaStreamPerThread;
        const SeamForm& f = seam_form();
        const int ra = std::max(*len_row_a, 1), rb = std::max(*len_row_b, 1);
        ScratchBuf dA, dB, dC;
        RT_TRY(scratch_alloc(dA, sizeof(double) * (size_t)ra * std::max(*len_column_a, 1), s));
        RT_TRY(scratch_alloc(dB, sizeof(double) * (size_t)rb * std::max(*len_column_b, 1), s));
        RT_TRY(scratch_alloc(dC, sizeof(double) * (size_t)m * n, s));
        if (*len_row_a > 0 && *len_column_a > 0)
            RT_CUDA_TRY(cudaMemcpy2DAsync(dA.p, sizeof(double) * ra,
                                          matr_a + (size_t)*start_column_a * *rows_a + *start_row_a,
                                          sizeof(double) * *rows_a, sizeof(double) * *len_row_a, *len_column_a,
                                          cudaMemcpyHostToDevice, s));
        if (*len_row_b > 0 && *len_column_b > 0)
            RT_CUDA_TRY(cudaMemcpy2DAsync(dB.p, sizeof(double) * rb,
                                          matr_b + (size_t)*start_column_b * *rows_b + *start_row_b,
                                          sizeof(double) * *rows_b, sizeof(double) * *len_row_b, *len_column_b,
                                          cudaMemcpyHostToDevice, s));
        double* cblk = matr_c + (size_t)*start_column_c * *rows_c + *start_row_c;
        RT_CUDA_TRY(cudaMemcpy2DAsync(dC.p, sizeof(double) * m, cblk, sizeof(double) * *rows_c, sizeof(double) * m,
                                      n, cudaMemcpyHostToDevice, s));
        if (f.form == RT_FORM_SPLIT) {
            // The product in the split form, then C <- alpha * P + beta * C in float64.
            ScratchBuf dP;
            RT_TRY(scratch_alloc(dP, sizeof(double) * (size_t)m * n, s));
            RT_TRY(rt_dgemm_split(oa, ob, m, n, k, dA.as<double>(), ra, dB.as<double>(), rb, dP.as<double>(), m,
                                  f.nslices, s));
            const int64_t total = (int64_t)m * n;
            axpby_block_kernel<<<(unsigned)std::min<int64_t>(ceil_div(total, 256), 4 * sm_count()), 256, 0, s>>>(
                dC.as<double>(), m, dP.as<double>(), m, n, *alpha, *beta);
            RT_TRY(check_launch("axpby_block_kernel"));
            RT_CUDA_TRY(cudaMemcpy2DAsync(cblk, sizeof(double) * *rows_c, dC.p, sizeof(double) * m,
                                          sizeof(double) * m, n, cudaMemcpyDeviceToHost, s));
            RT_CUDA_TRY(cudaStreamSynchronize(s));
            return RT_OK;
        }
        RT_TRY(rt_dgemm(oa, ob, m, n, k, *alpha, dA.as<double>(), ra, dB.as<double>(), rb, *beta, dC.as<double>(),
                        m, s));
        RT_CUDA_TRY(cudaMemcpy2DAsync(cblk, sizeof(double) * *rows_c, dC.p, sizeof(double) * m, sizeof(double) * m,
                                      n, cudaMemcpyDeviceToHost, s));
        RT_CUDA_TRY(cudaStreamSynchronize(s));
        return RT_OK;
    };
    if (run() != RT_OK) fprintf(stderr, "general_dgemm_f_: %s\n", rt_last_error());
}

void special_dgemm_f_01_(double* ten3_a, const int* x_a, const int* y_a, const int* z_a, const int* start_x_a,
                         const int* len_x_a, const int* i_y_a, const int* start_z_a, const int* len_z_a,
                         const double* matr_b, const int* rows_b, const int* columns_b, const int* start_row_b,
                         const int* len_row_b, const int* start_column_b, const int* len_column_b,
                         const double* alpha, const double* beta) {
    NvtxRange nvtx_range("special_dgemm_f_01_");
    rt::set_error(RT_OK, "");
    (void)i_y_a;  // the Fortran loops over every y-slice and never reads it
    auto run = [&]() -> rt_status {
        const int X = *x_a, Y = *y_a, Z = *z_a, lx = *len_x_a, lz = *len_z_a;
        RT_REQUIRE(X >= 0 && Y >= 0 && Z >= 0, "special_dgemm_f_01_: negative dimension");
        RT_REQUIRE(*start_x_a >= 0 && lx >= 0 && (int64_t)*start_x_a + lx <= X && *start_z_a >= 0 && lz >= 0 &&
                       (int64_t)*start_z_a + lz <= Z,
                   "special_dgemm_f_01_: block of ten3_a outside the tensor");
        RT_REQUIRE(*start_row_b >= 0 && *len_row_b >= 0 && (int64_t)*start_row_b + *len_row_b <= *rows_b &&
                       *start_column_b >= 0 && *len_column_b >= 0 &&
                       (int64_t)*start_column_b + *len_column_b <= *columns_b,
                   "special_dgemm_f_01_: block of matr_b outside the matrix");
        RT_REQUIRE(*len_row_b == lz && *len_column_b == lz,
                   "special_dgemm_f_01_: the block of matr_b must be len_z_a x len_z_a");
        RT_TRY(seam_check("special_dgemm_f_01_"));
        if ((int64_t)lx * Y * lz == 0) return RT_OK;
        cudaStream_t s = cudaStreamPerThread;
        const SeamForm& f = seam_form();
        const size_t blk_elems = (size_t)lx * Y * lz;
        ScratchBuf dT, dM;
        RT_TRY(scratch_alloc(dT, sizeof(double) * blk_elems, s));
        RT_TRY(scratch_alloc(dM, sizeof(double) * (size_t)lz * lz, s));
        // The block [lx, Y, lz] as a contiguous device tensor.
        cudaMemcpy3DParms up = {};
        up.srcPtr = make_cudaPitchedPtr(ten3_a, sizeof(double) * X, sizeof(double) * X, Y);
        up.srcPos = make_cudaPos(sizeof(double) * *start_x_a, 0, *start_z_a);
        up.dstPtr = make_cudaPitchedPtr(dT.p, sizeof(double) * lx, sizeof(double) * lx, Y);
        up.extent = make_cudaExtent(sizeof(double) * lx, Y, lz);
        up.kind = cudaMemcpyHostToDevice;
        RT_CUDA_TRY(cudaMemcpy3DAsync(&up, s));
        RT_CUDA_TRY(cudaMemcpy2DAsync(dM.p, sizeof(double) * lz,
                                      matr_b + (size_t)*start_column_b * *rows_b + *start_row_b,
                                      sizeof(double) * *rows_b, sizeof(double) * lz, lz, cudaMemcpyHostToDevice, s));
        RT_TRY(special_dgemm_01(dT.as<double>(), lx, Y, 0, lx, 0, lz, dM.as<double>(), lz, 0, 0, *alpha, *beta,
                                f.form, f.nslices, s));
        cudaMemcpy3DParms down = {};
        down.srcPtr = up.dstPtr;
        down.dstPtr = up.srcPtr;
        down.dstPos = up.srcPos;
        down.extent = up.extent;
        down.kind = cudaMemcpyDeviceToHost;
        RT_CUDA_TRY(cudaMemcpy3DAsync(&down, s));
        RT_CUDA_TRY(cudaStreamSynchronize(s));
        return RT_OK;
    };
    if (run() != RT_OK) fprintf(stderr, "special_dgemm_f_01_: %s\n", rt_last_error());
}

}  // extern "C"
