// davidson.cu - block Davidson eigensolver for the lowest roots of a
// symmetric operator, with vectors resident in HBM, plus the RI response
// operator A = diag(delta) + B_ov B_ov^T and the (ia|jb) block.
//
// The control flow follows the reference's davidson_solve
// (src/davidson.rs:48-266) and its helpers, including its quirks:
//   * maxspace += 3 (nroots - 1)                                  (:74)
//   * one starting vector; the space grows by the unconverged roots (:99-131)
//   * H_eff entries are float64 dot products, with the reference's fill order
//     (fill_heff, :327-390); Rayleigh-Ritz on the packed upper triangle (:144-145)
//   * residual r_k = A x_k - e_k x_k; converged when |de_k| < tol and
//     |r_k| < sqrt(tol)                                            (:176-200)
//   * the preconditioner shifts every root by e[0]                 (:63-70, :224)
//   * new directions are projected against the space in modified Gram-Schmidt
//     order, normalised, and dropped when |x|^2 <= lindep          (:235-245, :268-285)
//   * the restart test compares against the value set at the last fresh
//     start (the reference shadows max_dx_last at :259)
//   * in the non-fresh branch the new-vector count is taken before _qr (:112-118)
// The matrix-vector product is supplied by the caller on device pointers (the
// reference's `a_x` closure), one block of vectors per call.  Vector algebra
// is float64 on the device with fixed-order reductions; the subspace
// eigenproblem (order <= a few dozen) is solved in float64 on the host by
// Householder tridiagonalisation and implicit QR with Wilkinson shifts (Golub &
// Van Loan, Matrix Computations, Algorithms 8.3.1 and 8.3.3), with cyclic
// Jacobi rotations (8.5) as the fallback.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "rt_internal.cuh"

namespace rt {
namespace {

constexpr int kRedBlocks = 256;

// partial[b] = sum over this block's stride of x[i] * y[i]
__global__ void __launch_bounds__(256) dot_partial_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                                          int64_t n, double* __restrict__ partial) {
    __shared__ double red[8];
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(x[i], y[i], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < 8 ? red[threadIdx.x] : 0.0;
        for (int o = 4; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) partial[blockIdx.x] = t;
    }
}

// out[0] = sum(partial[0..nb)) in a fixed order.
__global__ void dot_final_kernel(const double* __restrict__ partial, int nb, double* __restrict__ out) {
    __shared__ double red[kRedBlocks];
    double v = threadIdx.x < nb ? partial[threadIdx.x] : 0.0;
    red[threadIdx.x] = v;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

// x -= (*c) * q
__global__ void axpy_dev_kernel(double* __restrict__ x, const double* __restrict__ q, const double* __restrict__ c,
                                int64_t n) {
    const double a = *c;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = fma(-a, q[i], x[i]);
}

// Column dots, several at once: partial[k * gridDim.x + b] = this block's share of
// sum_i A[i + k lda] * Bm[i + k ldb] for column k = blockIdx.y (lda = 0: one vector A
// against every column of Bm).  Fixed-order reduction, like dot_partial_kernel.
__global__ void __launch_bounds__(256) coldot_partial_kernel(const double* __restrict__ A, int64_t lda,
                                                             const double* __restrict__ Bm, int64_t ldb, int64_t n,
                                                             double* __restrict__ partial) {
    __shared__ double red[8];
    const int k = blockIdx.y;
    const double* a = A + (int64_t)k * lda;
    const double* b = Bm + (int64_t)k * ldb;
    double s = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s = fma(a[i], b[i], s);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = threadIdx.x < 8 ? red[threadIdx.x] : 0.0;
        for (int o = 4; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) partial[(int64_t)k * gridDim.x + blockIdx.x] = t;
    }
}

// X[:, k] -= c[k] * q for the nv columns of X (leading dimension ld).
__global__ void multi_axpy_kernel(double* __restrict__ X, int64_t ld, int nv, const double* __restrict__ q,
                                  const double* __restrict__ c, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double qi = q[i];
        for (int k = 0; k < nv; ++k) X[i + k * ld] = fma(-c[k], qi, X[i + k * ld]);
    }
}

// y = x / s  (host scalar; division as in the reference's `x /= norm`; y may equal x)
__global__ void div_kernel(double* y, const double* x, double s, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = x[i] / s;
}

// y = x / sqrt(*d2)  (a norm kept on the device; sqrt is correctly rounded, as on the host)
// (called in place: y may equal x)
__global__ void div_dev_sqrt_kernel(double* y, const double* x, const double* __restrict__ d2, int64_t n) {
    const double v = sqrt(*d2);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = x[i] / v;
}

// r = ax - e * x
__global__ void residual_kernel(double* __restrict__ r, const double* __restrict__ ax, const double* __restrict__ x,
                                double e, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = ax[i] - e * x[i];
}

// Preconditioner of davidson.rs:63-70: r_i / (hdiag_i - e), with |.| < 1e-8 replaced by 1e-8.
__global__ void precond_kernel(double* __restrict__ r, const double* __restrict__ hdiag, double e, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double h = hdiag[i] - e;
        if (fabs(h) < 1e-8) h = 1e-8;
        r[i] = r[i] / h;
    }
}

// hdiag[i] = delta[i] + sum_P B[i + nov*P]^2: the exact diagonal of diag(delta) + B B^T.
__global__ void response_diag_kernel(const double* __restrict__ B, const double* __restrict__ delta, int64_t nov,
                                     int naux, double* __restrict__ hdiag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nov; i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int P = 0; P < naux; ++P) {
            const double b = B[i + nov * (int64_t)P];
            s = fma(b, b, s);
        }
        hdiag[i] = delta[i] + s;
    }
}

// AX[:, v] += delta .* X[:, v]
__global__ void diag_add_kernel(double* __restrict__ AX, const double* __restrict__ delta,
                                const double* __restrict__ X, int64_t n, int nvec) {
    const int64_t total = n * nvec;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x)
        AX[i] = fma(delta[i % n], X[i], AX[i]);
}

struct VecOps {
    cudaStream_t s;
    double* partial = nullptr;  // kRedBlocks
    double* scalars = nullptr;  // scratch device scalars
    int grid = 0;

    rt_status dot(const double* x, const double* y, int64_t n, double* out_dev) {
        dot_partial_kernel<<<kRedBlocks, 256, 0, s>>>(x, y, n, partial);
        RT_TRY(check_launch("dot_partial_kernel"));
        dot_final_kernel<<<1, kRedBlocks, 0, s>>>(partial, kRedBlocks, out_dev);
        return check_launch("dot_final_kernel");
    }
    rt_status dot_host(const double* x, const double* y, int64_t n, double* out) {
        RT_TRY(dot(x, y, n, scalars));
        RT_CUDA_TRY(cudaMemcpyAsync(out, scalars, sizeof(double), cudaMemcpyDeviceToHost, s));
        RT_CUDA_TRY(cudaStreamSynchronize(s));
        return RT_OK;
    }
    rt_status norm_host(const double* x, int64_t n, double* out) {
        double d = 0.0;
        RT_TRY(dot_host(x, x, n, &d));
        *out = sqrt(d);
        return RT_OK;
    }
    // x -= (q . x) q   (one modified Gram-Schmidt step, scalar kept on the device)
    rt_status project_out(double* x, const double* q, int64_t n) {
        RT_TRY(dot(q, x, n, scalars + 1));
        axpy_dev_kernel<<<grid, 256, 0, s>>>(x, q, scalars + 1, n);
        return check_launch("axpy_dev_kernel");
    }
    rt_status divide(double* y, const double* x, double v, int64_t n) {
        div_kernel<<<grid, 256, 0, s>>>(y, x, v, n);
        return check_launch("div_kernel");
    }
    rt_status copy(double* y, const double* x, int64_t n) {
        RT_CUDA_TRY(cudaMemcpyAsync(y, x, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        return RT_OK;
    }
    // out_dev[k] = A[:, k] . Bm[:, k] for k < nv (lda = 0: the single vector A), each
    // reduced in a fixed order over kColBlocks partial sums.
    static constexpr int kColBlocks = 64;
    double* colpart = nullptr;  // kMaxCols * kColBlocks
    double* colout = nullptr;   // max(kMaxCols, ncolout) entries
    int ncolout = 0;
    static constexpr int kMaxCols = 64;
    rt_status coldots(const double* A, int64_t lda, const double* Bm, int64_t ldb, int nv, int64_t n,
                      double* out_dev) {
        for (int k0 = 0; k0 < nv; k0 += kMaxCols) {
            const int m = std::min(kMaxCols, nv - k0);
            coldot_partial_kernel<<<dim3(kColBlocks, m), 256, 0, s>>>(A + k0 * lda, lda, Bm + k0 * ldb, ldb, n,
                                                                      colpart);
            RT_TRY(check_launch("coldot_partial_kernel"));
            for (int k = 0; k < m; ++k) {
                dot_final_kernel<<<1, kRedBlocks, 0, s>>>(colpart + (int64_t)k * kColBlocks, kColBlocks,
                                                          out_dev + k0 + k);
                RT_TRY(check_launch("dot_final_kernel"));
            }
        }
        return RT_OK;
    }
    // Euclidean norms of the nv columns of X, read back with one synchronisation.
    rt_status norms_host(const double* X, int64_t ld, int nv, int64_t n, double* out) {
        if (nv <= 0) return RT_OK;
        RT_REQUIRE(nv <= ncolout, "rt_davidson_solve: too many columns for one norm batch");
        RT_TRY(coldots(X, ld, X, ld, nv, n, colout));
        std::vector<double> d(nv);
        RT_CUDA_TRY(cudaMemcpyAsync(d.data(), colout, sizeof(double) * nv, cudaMemcpyDeviceToHost, s));
        RT_CUDA_TRY(cudaStreamSynchronize(s));
        for (int k = 0; k < nv; ++k) out[k] = sqrt(d[k]);
        return RT_OK;
    }
    // X[:, k] -= (q . X[:, k]) q for k < nv: one modified Gram-Schmidt step of q
    // applied to every column, the coefficients kept on the device.
    rt_status project_out_many(double* X, int64_t ld, int nv, const double* q, int64_t n) {
        if (nv <= 0) return RT_OK;
        for (int k0 = 0; k0 < nv; k0 += kMaxCols) {
            const int m = std::min(kMaxCols, nv - k0);
            RT_TRY(coldots(q, 0, X + k0 * ld, ld, m, n, colout));
            multi_axpy_kernel<<<grid, 256, 0, s>>>(X + k0 * ld, ld, m, q, colout, n);
            RT_TRY(check_launch("multi_axpy_kernel"));
        }
        return RT_OK;
    }
};

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (column-major
// a, destroyed).  Eigenvalues ascending in w, eigenvectors in the columns of z.
void jacobi_eigh(int n, std::vector<double>& a, std::vector<double>& w, std::vector<double>& z) {
    z.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) z[(size_t)i * n + i] = 1.0;
    auto A = [&](int i, int j) -> double& { return a[(size_t)j * n + i]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i) (i == j ? diag : off) += A(i, j) * A(i, j);
        if (off <= 1e-30 * std::max(diag, 1e-300)) break;
        for (int p = 0; p < n - 1; ++p) {
            for (int q = p + 1; q < n; ++q) {
                const double apq = A(p, q);
                if (fabs(apq) < 1e-300) continue;
                const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
                for (int k = 0; k < n; ++k) {
                    const double akp = A(k, p), akq = A(k, q);
                    A(k, p) = c * akp - sn * akq;
                    A(k, q) = sn * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {
                    const double apk = A(p, k), aqk = A(q, k);
                    A(p, k) = c * apk - sn * aqk;
                    A(q, k) = sn * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double zkp = z[(size_t)p * n + k], zkq = z[(size_t)q * n + k];
                    z[(size_t)p * n + k] = c * zkp - sn * zkq;
                    z[(size_t)q * n + k] = sn * zkp + c * zkq;
                }
            }
        }
    }
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return A(x, x) < A(y, y); });
    w.resize(n);
    std::vector<double> zs((size_t)n * n);
    for (int k = 0; k < n; ++k) {
        w[k] = A(idx[k], idx[k]);
        // Fix the sign: largest-magnitude component positive.
        int imax = 0;
        for (int i = 1; i < n; ++i)
            if (fabs(z[(size_t)idx[k] * n + i]) > fabs(z[(size_t)idx[k] * n + imax])) imax = i;
        const double sg = z[(size_t)idx[k] * n + imax] < 0 ? -1.0 : 1.0;
        for (int i = 0; i < n; ++i) zs[(size_t)k * n + i] = sg * z[(size_t)idx[k] * n + i];
    }
    z.swap(zs);
}

// Eigen-decomposition of a symmetric n x n matrix (column-major a, destroyed):
// Householder reduction to tridiagonal form, then the implicit symmetric QR
// iteration with Wilkinson shifts (Golub & Van Loan, Matrix Computations,
// Algorithms 8.3.1 and 8.3.3), both accumulated into z.  About 9 n^3 flops
// against ~30 n^3 for cyclic Jacobi.  Same output convention as jacobi_eigh.
// Returns false if the QR iteration has not converged after 30 n steps.
bool qr_eigh(int n, std::vector<double>& a, std::vector<double>& w, std::vector<double>& z) {
    z.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) z[(size_t)i * n + i] = 1.0;
    auto A = [&](int i, int j) -> double& { return a[(size_t)j * n + i]; };
    auto Z = [&](int i, int j) -> double& { return z[(size_t)j * n + i]; };
    std::vector<double> v(n), p(n);
    // 1) A <- H_k A H_k with H_k = I - beta v v^T zeroing A[k+2:, k]; z <- z H_k.
    for (int k = 0; k + 2 < n; ++k) {
        double tail = 0.0;  // sum of squares below the subdiagonal
        for (int i = k + 2; i < n; ++i) tail += A(i, k) * A(i, k);
        if (tail == 0.0) continue;
        const double x0 = A(k + 1, k);
        const double xnorm = sqrt(x0 * x0 + tail);
        const double alpha = x0 >= 0.0 ? -xnorm : xnorm;  // sign chosen so that x0 - alpha does not cancel
        v[k + 1] = x0 - alpha;
        for (int i = k + 2; i < n; ++i) v[i] = A(i, k);
        const double beta = 1.0 / (xnorm * xnorm - alpha * x0);  // 2 / (v^T v)
        double vp = 0.0;
        for (int i = k + 1; i < n; ++i) {
            double t = 0.0;
            for (int j = k + 1; j < n; ++j) t += A(i, j) * v[j];
            p[i] = beta * t;
            vp += v[i] * p[i];
        }
        const double half = 0.5 * beta * vp;
        for (int i = k + 1; i < n; ++i) p[i] -= half * v[i];  // q = p - (beta/2)(v^T p) v
        for (int j = k + 1; j < n; ++j)
            for (int i = k + 1; i < n; ++i) A(i, j) -= v[i] * p[j] + p[i] * v[j];
        A(k + 1, k) = A(k, k + 1) = alpha;
        for (int i = k + 2; i < n; ++i) A(i, k) = A(k, i) = 0.0;
        for (int r = 0; r < n; ++r) {
            double t = 0.0;
            for (int j = k + 1; j < n; ++j) t += Z(r, j) * v[j];
            t *= beta;
            for (int j = k + 1; j < n; ++j) Z(r, j) -= t * v[j];
        }
    }
    std::vector<double> d(n), e(std::max(n, 1), 0.0);
    for (int i = 0; i < n; ++i) d[i] = A(i, i);
    for (int i = 0; i + 1 < n; ++i) e[i] = A(i + 1, i);
    // 2) Implicit QR steps on the trailing unreduced block [lo, hi].
    const double eps = 2.220446049250313e-16;
    int hi = n - 1, steps = 0;
    while (hi > 0) {
        if (fabs(e[hi - 1]) <= eps * (fabs(d[hi - 1]) + fabs(d[hi]))) {
            e[hi - 1] = 0.0;
            --hi;
            continue;
        }
        int lo = hi - 1;
        while (lo > 0 && fabs(e[lo - 1]) > eps * (fabs(d[lo - 1]) + fabs(d[lo]))) --lo;
        if (lo > 0) e[lo - 1] = 0.0;
        if (++steps > 30 * n) return false;
        // Wilkinson shift: the eigenvalue of the trailing 2 x 2 block nearer d[hi]
        const double dd = 0.5 * (d[hi - 1] - d[hi]);
        const double den = dd + copysign(hypot(dd, e[hi - 1]), dd);
        const double mu = den != 0.0 ? d[hi] - e[hi - 1] * e[hi - 1] / den : d[hi];
        double x = d[lo] - mu, bulge = e[lo];
        for (int k = lo; k < hi; ++k) {
            // Q = [c s; -s c] on rows/columns k, k+1 maps (x, bulge) to (r, 0).
            const double r = hypot(x, bulge);
            const double c = r != 0.0 ? x / r : 1.0, sn = r != 0.0 ? bulge / r : 0.0;
            if (k > lo) e[k - 1] = r;
            const double a0 = d[k], b0 = d[k + 1], o = e[k];
            d[k] = c * c * a0 + 2.0 * c * sn * o + sn * sn * b0;
            d[k + 1] = sn * sn * a0 - 2.0 * c * sn * o + c * c * b0;
            e[k] = c * sn * (b0 - a0) + (c * c - sn * sn) * o;
            if (k + 1 < hi) {  // the rotation pushes a bulge to (k+2, k)
                x = e[k];
                bulge = sn * e[k + 1];
                e[k + 1] = c * e[k + 1];
            }
            for (int rr = 0; rr < n; ++rr) {
                const double zk = Z(rr, k), zk1 = Z(rr, k + 1);
                Z(rr, k) = c * zk + sn * zk1;
                Z(rr, k + 1) = -sn * zk + c * zk1;
            }
        }
    }
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int x, int y) { return d[x] < d[y]; });
    w.resize(n);
    std::vector<double> zs((size_t)n * n);
    for (int k = 0; k < n; ++k) {
        w[k] = d[idx[k]];
        int imax = 0;  // sign: largest-magnitude component positive
        for (int i = 1; i < n; ++i)
            if (fabs(z[(size_t)idx[k] * n + i]) > fabs(z[(size_t)idx[k] * n + imax])) imax = i;
        const double sg = z[(size_t)idx[k] * n + imax] < 0 ? -1.0 : 1.0;
        for (int i = 0; i < n; ++i) zs[(size_t)k * n + i] = sg * z[(size_t)idx[k] * n + i];
    }
    z.swap(zs);
    return true;
}

// Rayleigh-Ritz eigensolver of the Davidson subspace: QR, with cyclic Jacobi
// as the fallback should the QR iteration not converge.
void subspace_eigh(int n, std::vector<double>& a, std::vector<double>& w, std::vector<double>& z) {
    std::vector<double> keep = a;
    if (!qr_eigh(n, a, w, z)) jacobi_eigh(n, keep, w, z);
}

}  // namespace

rt_status ri_response_matvec(const double* Bov, const double* delta, int64_t nov, int naux, const double* X,
                             double* AX, int nvec, int form, int nslices, cudaStream_t s);

}  // namespace rt

using namespace rt;

// Testing hook: the Davidson subspace eigensolver on a host matrix (no device work).
extern "C" rt_status rt_debug_symeig(int n, const double* a, double* w, double* z) {
    RT_REQUIRE(n >= 1 && a && w && z, "rt_debug_symeig: bad arguments");
    std::vector<double> m(a, a + (size_t)n * n), wv, zv;
    if (!qr_eigh(n, m, wv, zv)) {
        set_error(RT_ERR_NOT_CONVERGED, "rt_debug_symeig: QR iteration did not converge");
        return RT_ERR_NOT_CONVERGED;
    }
    std::copy(wv.begin(), wv.end(), w);
    std::copy(zv.begin(), zv.end(), z);
    return RT_OK;
}

extern "C" {

rt_status rt_davidson_solve(rt_matvec_fn a_x, void* ctx, const double* x0_1d, const double* hdiag, long long n,
                            const rt_davidson_params* params, int print_level, int* conv, double* e, double* x_out,
                            int* iterations, void* stream) {
    RT_REQUIRE(a_x && x0_1d && hdiag && params && conv && e && x_out, "rt_davidson_solve: null argument");
    RT_REQUIRE(n > 0 && n <= INT32_MAX, "rt_davidson_solve: n must be in 1..2^31-1");
    const int nroots = params->nroots;
    const double tol = params->tol, lindep = params->lindep;
    RT_REQUIRE(nroots >= 1, "rt_davidson_solve: nroots must be positive");
    if (n - nroots < 3) {  // davidson.rs:102-104
        set_error(RT_ERR_INVALID_ARG, "rt_davidson_solve: too many roots requested for the space (n - nroots < 3)");
        return RT_ERR_INVALID_ARG;
    }
    const int maxspace = params->maxspace + (nroots - 1) * 3;  // davidson.rs:74
    cudaStream_t s = (cudaStream_t)stream;
    // Room for the space plus one block of new vectors (at most 40 kept, :116-118).
    const int cap = maxspace + std::max(nroots, 40) + 1;
    ScratchBuf xsb, axb, xtb, wb, red;
    RT_TRY(scratch_alloc(xsb, sizeof(double) * (size_t)n * cap, s));
    RT_TRY(scratch_alloc(axb, sizeof(double) * (size_t)n * cap, s));
    RT_TRY(scratch_alloc(xtb, sizeof(double) * (size_t)n * cap, s));
    RT_TRY(scratch_alloc(wb, sizeof(double) * (size_t)n * std::max(2 * nroots, 2), s));
    RT_TRY(scratch_alloc(red, sizeof(double) * (kRedBlocks + 8), s));
    double* XS = xsb.as<double>();
    double* AXs = axb.as<double>();
    double* XT = xtb.as<double>();
    double* X0 = wb.as<double>();             // current Ritz vectors [n, nroots]
    double* AX0 = X0 + (size_t)n * nroots;    // their images
    ScratchBuf vb;
    RT_TRY(scratch_alloc(vb, sizeof(double) * (size_t)cap * cap, s));
    double* Vdev = vb.as<double>();
    // The Ritz coefficients go up through page-locked staging, so the upload does
    // not wait for the stream; `vdone` marks when the staging may be rewritten.
    double* Vpin = nullptr;
    RT_CUDA_TRY(cudaMallocHost(&Vpin, sizeof(double) * (size_t)cap * cap));
    cudaEvent_t vdone = nullptr;
    if (cudaEventCreateWithFlags(&vdone, cudaEventDisableTiming) != cudaSuccess) {
        cudaFreeHost(Vpin);
        RT_CUDA_TRY(cudaGetLastError());
    }
    struct Staging {
        double* p;
        cudaEvent_t e;
        ~Staging() {
            if (e) cudaEventSynchronize(e);
            if (e) cudaEventDestroy(e);
            if (p) cudaFreeHost(p);
        }
    } staging{Vpin, vdone};
    auto upload_v = [&](const double* V, int rows, int cols) -> rt_status {
        if ((int64_t)rows * cols == 0) return RT_OK;
        RT_CUDA_TRY(cudaEventSynchronize(vdone));
        std::copy(V, V + (size_t)rows * cols, Vpin);
        RT_CUDA_TRY(cudaMemcpyAsync(Vdev, Vpin, sizeof(double) * (size_t)rows * cols, cudaMemcpyHostToDevice, s));
        RT_CUDA_TRY(cudaEventRecord(vdone, s));
        return RT_OK;
    };
    // dst[n, cols] = src[n, rows] * V[rows, cols] with V uploaded (_gen_x0, davidson.rs:392-404).
    auto gen_x0 = [&](const double* src, int rows, int cols, double* dst) -> rt_status {
        if (cols == 0) return RT_OK;
        RT_TRY(rt_dgemm('N', 'N', (int)n, cols, rows, 1.0, src, (int)n, Vdev, rows, 0.0, dst, (int)n, s));
        return RT_OK;
    };
    VecOps ops{s, red.as<double>(), red.as<double>() + kRedBlocks, std::min<int>(4 * sm_count(), (int)ceil_div(n, 256))};
    if (ops.grid < 1) ops.grid = 1;
    ScratchBuf colb, gb;
    ops.ncolout = std::max(cap, (int)VecOps::kMaxCols);
    RT_TRY(scratch_alloc(colb, sizeof(double) * (size_t)(VecOps::kMaxCols * VecOps::kColBlocks + ops.ncolout), s));
    ops.colpart = colb.as<double>();
    ops.colout = ops.colpart + VecOps::kMaxCols * VecOps::kColBlocks;
    // X_new^T AX for fill_heff, at most cap x cap
    RT_TRY(scratch_alloc(gb, sizeof(double) * (size_t)cap * cap, s));
    std::vector<double> ghost((size_t)cap * cap);
    auto col = [&](double* base, int j) { return base + (size_t)j * n; };

    // Modified Gram-Schmidt of the columns of src (count m) into dst; returns the kept count.
    // First an optimistic pass that keeps every vector: each norm stays on the device
    // and the norms are read back once.  If all pass the reference's test, the result
    // is the one the vector-by-vector pass below gives (same dot kernel, same
    // correctly rounded sqrt); otherwise that pass runs again from src.
    auto qr = [&](double* dst, const double* src, int m, int* kept) -> rt_status {
        if (m > 0 && m <= ops.ncolout) {
            for (int i = 0; i < m; ++i) {
                double* xi = col(dst, i);
                if (xi != src + (size_t)i * n) RT_TRY(ops.copy(xi, src + (size_t)i * n, n));
                for (int j = 0; j < i; ++j) RT_TRY(ops.project_out(xi, col(dst, j), n));
                RT_TRY(ops.dot(xi, xi, n, ops.colout + i));
                div_dev_sqrt_kernel<<<ops.grid, 256, 0, s>>>(xi, xi, ops.colout + i, n);
                RT_TRY(check_launch("div_dev_sqrt_kernel"));
            }
            std::vector<double> d2(m);
            RT_CUDA_TRY(cudaMemcpyAsync(d2.data(), ops.colout, sizeof(double) * m, cudaMemcpyDeviceToHost, s));
            RT_CUDA_TRY(cudaStreamSynchronize(s));
            bool all = true;
            for (int i = 0; i < m; ++i) {
                const double norm = sqrt(d2[i]);
                all = all && norm * norm > lindep;
            }
            if (all) {
                *kept = m;
                return RT_OK;
            }
        }
        int nv = 0;
        for (int i = 0; i < m; ++i) {
            double* xi = col(dst, nv);
            if (xi != src + (size_t)i * n) RT_TRY(ops.copy(xi, src + (size_t)i * n, n));
            for (int j = 0; j < nv; ++j) RT_TRY(ops.project_out(xi, col(dst, j), n));
            double norm = 0.0;
            RT_TRY(ops.norm_host(xi, n, &norm));
            if (norm * norm > lindep) {
                RT_TRY(ops.divide(xi, xi, norm, n));
                ++nv;
            }
        }
        *kept = nv;
        return RT_OK;
    };

    // x0 = [x0_1d]
    RT_TRY(ops.copy(XT, x0_1d, n));
    int nx0 = 1;
    double* x0src = XT;
    bool fresh = true;
    int xtlen = 0, nxt = 0, space = 0;
    std::vector<double> ev, elast;
    std::vector<double> heff;  // space x space, column-major
    std::vector<double> vmat, vlast;  // [space, nroots_current]
    std::vector<int> convv(nroots, 0), convlast(nroots, 0);
    double max_dx_last = 1e9;
    int nroots_current = 0;
    int icyc = 0;
    std::vector<double> dxn, de;
    for (icyc = 0; icyc < params->maxcyc; ++icyc) {
        if (fresh) {
            space = 0;
            int kept = 0;
            // _qr(x0): the new vectors go straight into the subspace storage.
            RT_TRY(qr(XS, x0src, nx0, &kept));
            xtlen = kept;
            nxt = kept;
            if (xtlen == 0) {
                set_error(RT_ERR_NOT_CONVERGED, "rt_davidson_solve: no linearly independent start vector");
                return RT_ERR_NOT_CONVERGED;
            }
            max_dx_last = 1e9;
            heff.clear();
        } else {
            xtlen = nxt;
            int kept = nxt;
            if (nxt > 1) {
                RT_TRY(qr(col(XS, space), XT, nxt, &kept));
                if (kept > 40) kept = 40;
            } else if (nxt == 1) {
                RT_TRY(ops.copy(col(XS, space), XT, n));
            }
            nxt = kept;
            if (nxt != xtlen) {
                // The reference then indexes past its H_eff (davidson.rs:112-118, 133-146);
                // stop with an error instead.
                set_error(RT_ERR_NOT_CONVERGED,
                          "rt_davidson_solve: orthogonalisation dropped a new vector (reference behaviour undefined)");
                return RT_ERR_NOT_CONVERGED;
            }
        }
        // A x for the new block
        RT_TRY(a_x(col(XS, space), col(AXs, space), nxt, n, ctx, stream));
        const int head = space;
        space += xtlen;
        elast = ev;
        vlast = vmat;
        convlast = convv;
        // fill_heff (davidson.rs:327-390)
        {
            const int row0 = head, row1 = space;
            std::vector<double> hn((size_t)space * space, 0.0);
            if (!fresh)
                for (int j = 0; j < head; ++j)
                    for (int i = 0; i < head; ++i) hn[(size_t)j * space + i] = heff[(size_t)j * head + i];
            // The reference's loops (davidson.rs:345-380) leave H(i, j) = x_max(i,j) . ax_min(i,j)
            // for every pair with a new index; all of those are entries of
            // G = X_new^T AX[:, 0:space], formed by one GEMM and read back once.
            const int nnewc = row1 - row0;
            RT_TRY(rt_dgemm('T', 'N', nnewc, space, (int)n, 1.0, col(XS, row0), (int)n, AXs, (int)n, 0.0,
                            gb.as<double>(), nnewc, s));
            RT_CUDA_TRY(cudaMemcpyAsync(ghost.data(), gb.p, sizeof(double) * (size_t)nnewc * space,
                                        cudaMemcpyDeviceToHost, s));
            RT_CUDA_TRY(cudaStreamSynchronize(s));
            auto G = [&](int a, int b) { return ghost[(size_t)b * nnewc + (a - row0)]; };  // x_a . ax_b, a new
            for (int i = 0; i < row1; ++i)
                for (int j = std::max(i, row0); j < row1; ++j) {
                    const double v = G(j, i);  // j = max(i, j) is new
                    hn[(size_t)j * space + i] = v;
                    hn[(size_t)i * space + j] = v;
                }
            heff.swap(hn);
        }
        // Rayleigh-Ritz
        std::vector<double> a = heff, w, z;
        subspace_eigh(space, a, w, z);
        nroots_current = std::min(space, nroots);
        ev.assign(w.begin(), w.begin() + nroots_current);
        vmat.assign(z.begin(), z.begin() + (size_t)space * nroots_current);
        // x0 = XS v, ax0 = AX v  (_gen_x0, davidson.rs:392-404)
        RT_TRY(upload_v(vmat.data(), space, nroots_current));
        RT_TRY(gen_x0(XS, space, nroots_current, X0));
        RT_TRY(gen_x0(AXs, space, nroots_current, AX0));
        dxn.assign(nroots_current, 0.0);
        de.assign(nroots_current, 0.0);
        bool all_conv = true;
        for (int k = 0; k < nroots; ++k) convv[k] = 0;
        for (int k = 0; k < nroots_current; ++k) {
            de[k] = k < (int)elast.size() ? ev[k] - elast[k] : ev[k];
            residual_kernel<<<ops.grid, 256, 0, s>>>(col(XT, k), col(AX0, k), col(X0, k), ev[k], n);
            RT_TRY(check_launch("residual_kernel"));
        }
        RT_TRY(ops.norms_host(XT, n, nroots_current, n, dxn.data()));
        for (int k = 0; k < nroots_current; ++k) convv[k] = fabs(de[k]) < tol && dxn[k] < sqrt(tol);
        for (int k = 0; k < nroots; ++k) all_conv = all_conv && convv[k];
        const double max_dx = *std::max_element(dxn.begin(), dxn.end());
        if (print_level > 0)
            fprintf(stderr, "davidson step %d |r|=%.3e e0=%.12f space=%d\n", icyc, max_dx, ev[0], space);
        if (all_conv) break;
        if (max_dx > 1.0 && max_dx / max_dx_last > 3.0 && space > nroots + 2) {
            // Restore the previous Ritz vectors and restart (davidson.rs:210-217).
            const int nl = (int)(vlast.size() / std::max(head, 1));
            RT_TRY(upload_v(vlast.data(), head, nl));
            RT_TRY(gen_x0(XS, head, nl, XT));
            x0src = XT;
            nx0 = nl;
            fresh = true;
            continue;
        }
        // Precondition, normalise and project the residuals (davidson.rs:222-245).
        // Each vector's steps depend only on that vector, so the norms of a phase are
        // formed together and read back with one synchronisation.
        int nnew = 0;
        for (int k = 0; k < nroots_current; ++k) {
            if (dxn[k] * dxn[k] > lindep) {
                double* t = col(XT, nnew);
                if (t != col(XT, k)) RT_TRY(ops.copy(t, col(XT, k), n));
                precond_kernel<<<ops.grid, 256, 0, s>>>(t, hdiag, ev[0], n);
                RT_TRY(check_launch("precond_kernel"));
                ++nnew;
            }
        }
        std::vector<double> nrm(std::max(nnew, 1));
        RT_TRY(ops.norms_host(XT, n, nnew, n, nrm.data()));
        for (int k = 0; k < nnew; ++k) RT_TRY(ops.divide(col(XT, k), col(XT, k), nrm[k], n));
        // Modified Gram-Schmidt against the subspace, in the reference's order
        // (subspace vector i outer, new vectors inner).
        for (int i = 0; i < space; ++i) RT_TRY(ops.project_out_many(XT, n, nnew, col(XS, i), n));
        RT_TRY(ops.norms_host(XT, n, nnew, n, nrm.data()));
        int kept = 0;
        for (int k = 0; k < nnew; ++k) {
            const double norm = nrm[k];
            if (norm * norm > lindep) {
                RT_TRY(ops.divide(col(XT, kept), col(XT, k), norm, n));
                ++kept;
            }
        }
        nxt = kept;
        if (nxt == 0) {
            for (int k = 0; k < nroots_current; ++k) convv[k] = convv[k] || dxn[k] < sqrt(tol);
            break;
        }
        fresh = space + nroots > maxspace;
        if (fresh) {
            // Fresh start from the current Ritz vectors (x0 = XS v).
            RT_TRY(ops.copy(XT, X0, (int64_t)n * nroots_current));
            x0src = XT;
            nx0 = nroots_current;
        }
    }
    for (int k = 0; k < nroots; ++k) {
        conv[k] = convv[k];
        e[k] = k < (int)ev.size() ? ev[k] : 0.0;
    }
    RT_CUDA_TRY(cudaMemcpyAsync(x_out, X0, sizeof(double) * (size_t)n * nroots_current, cudaMemcpyDeviceToDevice, s));
    if (iterations) *iterations = icyc + 1;
    RT_CUDA_TRY(cudaStreamSynchronize(s));
    return RT_OK;
}

namespace {
struct ResponseCtx {
    const double* Bov;
    const double* delta;
    int64_t nov;
    int naux, form, nslices;
};
rt_status response_cb(const double* x, double* ax, int nvec, long long n, void* ctx, void* stream) {
    const ResponseCtx* c = static_cast<const ResponseCtx*>(ctx);
    return ri_response_matvec(c->Bov, c->delta, n, c->naux, x, ax, nvec, c->form, c->nslices, (cudaStream_t)stream);
}
}  // namespace

rt_status rt_davidson_ri_response(const double* Bov, const double* delta, long long nov, int naux, int form,
                                  int nslices, const double* x0_1d, const rt_davidson_params* params, int print_level,
                                  int* conv, double* e, double* x_out, int* iterations, void* stream) {
    RT_REQUIRE(form == RT_FORM_FP64 || (form == RT_FORM_SPLIT && nslices >= 3 && nslices <= 8),
               "rt_davidson_ri_response: bad form/nslices");
    RT_REQUIRE(nov > 0 && Bov && delta && x0_1d, "rt_davidson_ri_response: bad argument");
    cudaStream_t s = (cudaStream_t)stream;
    ScratchBuf hb;
    RT_TRY(scratch_alloc(hb, sizeof(double) * (size_t)nov, s));
    response_diag_kernel<<<4 * sm_count(), 256, 0, s>>>(Bov, delta, nov, naux, hb.as<double>());
    RT_TRY(check_launch("response_diag_kernel"));
    ResponseCtx c{Bov, delta, nov, naux, form, nslices};
    return rt_davidson_solve(response_cb, &c, x0_1d, hb.as<double>(), nov, params, print_level, conv, e, x_out,
                             iterations, stream);
}

rt_status rt_ri_response_matvec(const double* Bov, const double* delta, long long nov, int naux, const double* X,
                                double* AX, int nvec, int form, int nslices, void* stream) {
    RT_REQUIRE(nov >= 0 && naux >= 0 && nvec >= 0, "rt_ri_response_matvec: negative dimension");
    RT_REQUIRE(nov <= INT32_MAX, "rt_ri_response_matvec: nov above 2^31-1");
    return ri_response_matvec(Bov, delta, nov, naux, X, AX, nvec, form, nslices, (cudaStream_t)stream);
}

rt_status rt_ri_iajb(const double* Bov, long long nov, int naux, double* M, int form, int nslices, void* stream) {
    RT_REQUIRE(nov >= 0 && naux >= 0, "rt_ri_iajb: negative dimension");
    RT_REQUIRE(nov <= INT32_MAX, "rt_ri_iajb: nov above 2^31-1");
    if (nov == 0) return RT_OK;
    if (form == RT_FORM_SPLIT)
        return rt_dgemm_split('N', 'T', (int)nov, (int)nov, naux, Bov, (int)nov, Bov, (int)nov, M, (int)nov, nslices,
                              stream);
    return rt_dgemm('N', 'T', (int)nov, (int)nov, naux, 1.0, Bov, (int)nov, Bov, (int)nov, 0.0, M, (int)nov, stream);
}

}  // extern "C"

namespace rt {

rt_status ri_response_matvec(const double* Bov, const double* delta, int64_t nov, int naux, const double* X,
                             double* AX, int nvec, int form, int nslices, cudaStream_t s) {
    if (nov == 0 || nvec == 0) return RT_OK;
    if (naux == 0) {
        RT_CUDA_TRY(cudaMemsetAsync(AX, 0, sizeof(double) * (size_t)nov * nvec, s));
    } else {
        ScratchBuf tb;
        RT_TRY(scratch_alloc(tb, sizeof(double) * (size_t)naux * nvec, s));
        double* T = tb.as<double>();
        if (form == RT_FORM_SPLIT) {
            RT_TRY(rt_dgemm_split('T', 'N', naux, nvec, (int)nov, Bov, (int)nov, X, (int)nov, T, naux, nslices, s));
            RT_TRY(rt_dgemm_split('N', 'N', (int)nov, nvec, naux, Bov, (int)nov, T, naux, AX, (int)nov, nslices, s));
        } else {
            RT_TRY(rt_dgemm('T', 'N', naux, nvec, (int)nov, 1.0, Bov, (int)nov, X, (int)nov, 0.0, T, naux, s));
            RT_TRY(rt_dgemm('N', 'N', (int)nov, nvec, naux, 1.0, Bov, (int)nov, T, naux, 0.0, AX, (int)nov, s));
        }
    }
    diag_add_kernel<<<4 * sm_count(), 256, 0, s>>>(AX, delta, X, nov, nvec);
    return check_launch("diag_add_kernel");
}

}  // namespace rt
