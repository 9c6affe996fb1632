// symeig.cu - float64 symmetric eigensolver on the device, and the SCF-side
// routines built on it: lapack_dsyev, lapack_power and lapack_dspgvx
// (src/matrix/matrix_blas_lapack.rs:775-797, 1004-1064, 1096-1147).
//
// Method (Golub & Van Loan, Matrix Computations, 4th ed.):
//  1. Householder reduction to tridiagonal form A = Q T Q^T (Algorithm 8.3.1)
//     on the device, lower triangle, the trailing block kept fully symmetric.
//     Per column k there are two launches:
//       * one CTA: w = p - (tau/2)(p.v) v, the rank-2 update of the next
//         column, and that column's Householder vector;
//       * one warp per remaining column: the rank-2 update A -= v w^T + w v^T
//         fused with the next step's product p' = tau' A' v' (one pass over the
//         trailing block per step).
//     The update uses separately rounded products, so the block stays exactly
//     symmetric.
//  2. Q formed on the device by backward accumulation of the reflectors.
//  3. The implicit symmetric QR iteration with Wilkinson shifts on (d, e)
//     (Algorithm 8.3.3) on the host: O(n) per sweep; its Givens rotations are
//     recorded and
//  4. applied to the rows of Q on the device, 32 sweeps per pass in a systolic
//     warp per row (lane j applies sweep j, columns passed lane to lane).
//  5. Eigenvalues sorted ascending; each eigenvector's largest-magnitude
//     component made positive (LAPACK fixes no sign either).
// All reductions have a fixed order, so results are bitwise reproducible.
#include <math.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "rt_internal.cuh"

namespace rt {
namespace {

constexpr int kHouseThreads = 1024;

// Fixed-order sum over a CTA of kHouseThreads threads (every thread gets it).
__device__ __forceinline__ double cta_sum(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    return t;
}

// Householder vector of x = A[c+1 .. n-1, c] (length m = n - c - 1):
//   (I - tau v v^T) x = beta e_1,  v[0] = 1,  beta = -sign(x0) ||x||.
// Writes v to vout[0..m), tau, d[c] = A[c, c] and e[c] = beta.  A zero tail
// gives tau = 0 (no reflection) and e[c] = x0.
__device__ void house_body(const double* __restrict__ A, int64_t n, int64_t c, double* __restrict__ vout,
                           double* __restrict__ tau, double* __restrict__ d, double* __restrict__ e, double* red) {
    const int64_t m = n - c - 1;
    const double* x = A + c * n + c + 1;
    double t = 0.0;
    for (int64_t i = 1 + threadIdx.x; i < m; i += blockDim.x) t = fma(x[i], x[i], t);
    const double tail = cta_sum(t, red);
    const double x0 = x[0];
    if (tail == 0.0) {
        for (int64_t i = threadIdx.x; i < m; i += blockDim.x) vout[i] = i == 0 ? 1.0 : 0.0;
        if (threadIdx.x == 0) {
            tau[c] = 0.0;
            d[c] = A[c * n + c];
            e[c] = x0;
        }
        return;
    }
    const double xnorm = sqrt(fma(x0, x0, tail));
    const double beta = x0 >= 0.0 ? -xnorm : xnorm;
    const double scale = 1.0 / (x0 - beta);
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) vout[i] = i == 0 ? 1.0 : x[i] * scale;
    if (threadIdx.x == 0) {
        tau[c] = (beta - x0) / beta;
        d[c] = A[c * n + c];
        e[c] = beta;
    }
}

__global__ void __launch_bounds__(kHouseThreads) house_kernel(const double* A, int64_t n, int64_t c, double* vout,
                                                              double* tau, double* d, double* e) {
    __shared__ double red[32];
    house_body(A, n, c, vout, tau, d, e, red);
}

// p = tau_c * A22 v for the trailing block of column c (rows/cols c+1..n-1), one
// warp per column (the block is symmetric, so column j dotted with v is p_j).
__global__ void __launch_bounds__(256) symv_kernel(const double* __restrict__ A, int64_t n, int64_t c,
                                                   const double* __restrict__ v, const double* __restrict__ tau,
                                                   double* __restrict__ p) {
    const int64_t m = n - c - 1;
    const int lane = threadIdx.x & 31;
    const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= m) return;
    const double* col = A + (c + 1 + j) * n + c + 1;
    double t = 0.0;
    for (int64_t i = lane; i < m; i += 32) t = fma(col[i], v[i], t);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) p[j] = tau[c] * t;
}

// Step c, one CTA: w = p - (tau/2)(p.v) v; update column 0 of the trailing block
// (A column c+1, rows c+1..n-1); then, if column c+1 has a tail to reduce, its
// Householder vector into vnext (and tau, d, e of column c+1).
__global__ void __launch_bounds__(kHouseThreads) step_kernel(double* __restrict__ A, int64_t n, int64_t c,
                                                             const double* __restrict__ v,
                                                             const double* __restrict__ p, double* __restrict__ w,
                                                             double* __restrict__ vnext, double* tau, double* d,
                                                             double* e) {
    __shared__ double red[32];
    const int64_t m = n - c - 1;
    double t = 0.0;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) t = fma(p[i], v[i], t);
    const double pv = cta_sum(t, red);
    const double h = 0.5 * tau[c] * pv;
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) w[i] = fma(-h, v[i], p[i]);
    __syncthreads();
    double* col = A + (c + 1) * n + c + 1;
    const double v0 = v[0], w0 = w[0];
    for (int64_t i = threadIdx.x; i < m; i += blockDim.x) col[i] -= __dadd_rn(__dmul_rn(v[i], w0), __dmul_rn(w[i], v0));
    __syncthreads();
    if (m >= 3) house_body(A, n, c + 1, vnext, tau, d, e, red);  // column c+1 has a tail below its subdiagonal
}

// Step c, one warp per column j = 1..m-1 of the trailing block: the rank-2
// update of the column, and (when column c+1 is reduced next) the next product
// p'[j-1] = tau' * sum_{i >= 1} A22[i, j] v'[i-1].
__global__ void __launch_bounds__(256) update_symv_kernel(double* __restrict__ A, int64_t n, int64_t c,
                                                          const double* __restrict__ v,
                                                          const double* __restrict__ w,
                                                          const double* __restrict__ vnext,
                                                          const double* __restrict__ tau, double* __restrict__ pnext,
                                                          int want_next) {
    const int64_t m = n - c - 1;
    const int lane = threadIdx.x & 31;
    const int64_t j = 1 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (j >= m) return;
    double* col = A + (c + 1 + j) * n + c + 1;
    const double vj = v[j], wj = w[j];
    double t = 0.0;
    for (int64_t i = lane; i < m; i += 32) {
        const double a = col[i] - __dadd_rn(__dmul_rn(v[i], wj), __dmul_rn(w[i], vj));
        col[i] = a;
        if (i >= 1) t = fma(a, vnext[i - 1], t);
    }
    if (want_next) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) pnext[j - 1] = tau[c + 1] * t;
    }
}

// Backward accumulation, step c: Q[c+1:, c+1:] -= tau_c v (v^T Q[c+1:, c+1:]),
// with v stored in V column c (rows c+1..n-1).  One warp per column.
__global__ void __launch_bounds__(256) form_q_kernel(double* __restrict__ Q, const double* __restrict__ V, int64_t n,
                                                     int64_t c, const double* __restrict__ tau) {
    const int64_t m = n - c - 1;
    const int lane = threadIdx.x & 31;
    const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= m) return;
    const double tc = tau[c];
    if (tc == 0.0) return;
    double* col = Q + (c + 1 + j) * n + c + 1;
    const double* v = V + c * n + c + 1;
    double t = 0.0;
    for (int64_t i = lane; i < m; i += 32) t = fma(v[i], col[i], t);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    const double y = tc * t;
    for (int64_t i = lane; i < m; i += 32) col[i] = fma(-y, v[i], col[i]);
}

__global__ void identity_kernel(double* Q, int64_t n) {
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * n;
         idx += (int64_t)gridDim.x * blockDim.x)
        Q[idx] = (idx % n) == (idx / n) ? 1.0 : 0.0;
}

// A[i, j] = A[j, i] for i < j (LAPACK 'L': only the lower triangle is read).
__global__ void lower_to_full_kernel(const double* __restrict__ in, double* __restrict__ out, int64_t n) {
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % n, j = idx / n;
        out[idx] = i >= j ? in[idx] : in[j + n * i];
    }
}

// Recorded Givens sweeps of the QR iteration: sweep s rotates columns
// (k, k+1) for k = lo[s] .. hi[s]-1 with (c, s) at rot[first[s] + k - lo[s]]:
//   z_k <- c z_k + s z_{k+1},   z_{k+1} <- -s z_k + c z_{k+1},
// applied to every row of Z.
//
// Systolic form: 32 consecutive sweeps per pass, one warp per row, lane j
// applying sweep s0 + j.  At step t lane j rotates columns (t - 2j, t - 2j + 1):
// it holds column t - 2j, receives column t - 2j + 1 from lane j - 1 (which
// finished it in step t - 1) and hands the finished column t - 2j to lane j + 1.
// Lane 0 takes the row's next column, lane 31 returns column t - 62, which every
// sweep of the pass has finished.  The order of the rotations on each column
// pair is that of the sweeps, so the result is the sequential one.  Columns pass
// through shared-memory tiles of 32 columns x ROWS rows (coalesced loads and
// stores), and each 32-step chunk's rotations are staged in shared memory, an
// identity where a sweep has no rotation, so the steps have no branches.  The
// FP64 work is spread over 32 lanes per row.
constexpr int kSysRows = 16;

__global__ void __launch_bounds__(kSysRows * 32) rot_systolic_kernel(double* __restrict__ Z, int64_t n,
                                                                     const int* __restrict__ lo,
                                                                     const int* __restrict__ hi,
                                                                     const int64_t* __restrict__ first,
                                                                     const double2* __restrict__ rot, int s0,
                                                                     int nsw) {
    __shared__ double tin[kSysRows][33];
    __shared__ double tout[kSysRows][33];
    __shared__ double2 prm[32][33];
    __shared__ int slo[32], shi[32];
    __shared__ int64_t sfirst[32];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (tid < 32) {
        const bool on = tid < nsw;
        slo[tid] = on ? lo[s0 + tid] : 1 << 30;
        shi[tid] = on ? hi[s0 + tid] : -1;
        sfirst[tid] = on ? first[s0 + tid] : 0;
    }
    __syncthreads();
    int cmin = 1 << 30, cmax = -1;
    for (int j = 0; j < nsw; ++j) {
        cmin = min(cmin, slo[j]);
        cmax = max(cmax, shi[j]);
    }
    const int64_t row0 = (int64_t)blockIdx.x * kSysRows;
    double lower = 0.0, out = 0.0;
    // tile element (row w', column offset i) is moved by thread (w' + kSysRows * i) % blockDim
    const int mw = tid % kSysRows, mi = tid / kSysRows;  // mi in 0..31
    const bool mrow = row0 + mw < n;
    for (int T = cmin - 1; T <= cmax + 62; T += 32) {
        {
            const int c = T + 1 + mi;
            tin[mw][mi] = (mrow && c >= cmin && c <= cmax) ? Z[row0 + mw + (int64_t)c * n] : 0.0;
        }
        for (int q = tid; q < 32 * 32; q += kSysRows * 32) {
            const int j = q >> 5, u = q & 31;
            const int k = T + u - 2 * j;
            prm[j][u] = (k >= slo[j] && k < shi[j]) ? rot[sfirst[j] + (k - slo[j])] : make_double2(1.0, 0.0);
        }
        __syncthreads();
#pragma unroll 8
        for (int u = 0; u < 32; ++u) {
            double upper = __shfl_up_sync(0xffffffffu, out, 1);
            if (lane == 0) upper = tin[w][u];
            const double2 cs = prm[lane][u];
            out = fma(cs.x, lower, cs.y * upper);
            lower = fma(cs.x, upper, -cs.y * lower);
            if (lane == 31) tout[w][u] = out;
        }
        __syncthreads();
        {
            const int c = T - 62 + mi;
            if (mrow && c >= cmin && c <= cmax) Z[row0 + mw + (int64_t)c * n] = tout[mw][mi];
        }
    }
}

// out[:, j] = sign_j Z[:, perm[j]] with sign_j making the column's
// largest-magnitude entry (first on ties) positive.  One warp per column.
__global__ void __launch_bounds__(256) sort_sign_kernel(const double* __restrict__ Z, double* __restrict__ out,
                                                        int64_t n, const int* __restrict__ perm) {
    const int lane = threadIdx.x & 31;
    const int64_t j = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (j >= n) return;
    const double* z = Z + (int64_t)perm[j] * n;
    double best = -1.0;
    int64_t bi = 0;
    for (int64_t i = lane; i < n; i += 32) {
        const double a = fabs(z[i]);
        if (a > best) { best = a; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    const double sg = z[bi] < 0.0 ? -1.0 : 1.0;
    double* o = out + j * n;
    for (int64_t i = lane; i < n; i += 32) o[i] = sg * z[i];
}

// Implicit symmetric QR with Wilkinson shifts on the tridiagonal (d, e),
// recording every sweep's rotations.  Returns false without convergence in 30 n
// sweeps.  Rotations follow the convention of rot_systolic_kernel.
struct Sweeps {
    std::vector<int> lo, hi;
    std::vector<int64_t> first;
    std::vector<double2> rot;
};

// sqrt(x^2 + y^2), through hypot only where the squares could overflow or underflow.
inline double norm2(double x, double y) {
    const double ax = fabs(x), ay = fabs(y), m = ax > ay ? ax : ay;
    if (m < 1e150 && (m > 1e-150 || m == 0.0)) return sqrt(x * x + y * y);
    return hypot(x, y);
}

bool tridiag_qr(int n, std::vector<double>& d, std::vector<double>& e, Sweeps& sw) {
    const double eps = 2.220446049250313e-16;
    sw.rot.reserve((size_t)n * (size_t)n);
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
        sw.lo.push_back(lo);
        sw.hi.push_back(hi);
        sw.first.push_back((int64_t)sw.rot.size());
        for (int k = lo; k < hi; ++k) {
            // [c s; -s c] on rows/columns k, k+1 maps (x, bulge) to (r, 0).
            const double r = norm2(x, bulge);
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
            sw.rot.push_back(make_double2(c, sn));
        }
    }
    return true;
}

}  // namespace

// Eigen-decomposition of the symmetric n x n device matrix whose lower triangle
// is in A (column-major, leading dimension n): eigenvalues ascending into w
// (device, n) and orthonormal eigenvectors into the columns of V (device,
// n x n; may alias A).  Scratch: 3 n^2 + O(n) doubles.
rt_status symeig_device(int n_, const double* A, double* w, double* V, cudaStream_t s) {
    const int64_t n = n_;
    RT_REQUIRE(n >= 1, "symeig: empty matrix");
    ScratchBuf wa, qa, va, vec;
    RT_TRY(scratch_alloc(wa, sizeof(double) * (size_t)(n * n), s));
    RT_TRY(scratch_alloc(qa, sizeof(double) * (size_t)(n * n), s));
    RT_TRY(scratch_alloc(va, sizeof(double) * (size_t)(n * n), s));
    RT_TRY(scratch_alloc(vec, sizeof(double) * (size_t)(8 * n + 8), s));
    double* W = wa.as<double>();  // the matrix being reduced
    double* Q = qa.as<double>();
    double* Vst = va.as<double>();  // reflector k in column k, rows k+1..n-1
    double* tau = vec.as<double>();
    double* d = tau + n;
    double* e = d + n;
    double* p = e + n;
    double* wv = p + n;
    const unsigned g1 = (unsigned)std::min<int64_t>(ceil_div(n * n, 256), 8 * sm_count());
    lower_to_full_kernel<<<g1, 256, 0, s>>>(A, W, n);
    RT_TRY(check_launch("lower_to_full_kernel"));
    RT_CUDA_TRY(cudaMemsetAsync(Vst, 0, sizeof(double) * (size_t)(n * n), s));
    RT_CUDA_TRY(cudaMemsetAsync(tau, 0, sizeof(double) * (size_t)(3 * n), s));
    // Reflectors for columns 0 .. n-3; reflector c is written straight into
    // its storage column (Vst column c, rows c+1..n-1).
    auto vcol = [&](int64_t c) { return Vst + c * n + c + 1; };
    if (n >= 3) {
        house_kernel<<<1, kHouseThreads, 0, s>>>(W, n, 0, vcol(0), tau, d, e);
        RT_TRY(check_launch("house_kernel"));
        symv_kernel<<<(unsigned)ceil_div((n - 1) * 32, 256), 256, 0, s>>>(W, n, 0, vcol(0), tau, p);
        RT_TRY(check_launch("symv_kernel"));
        for (int64_t c = 0; c + 2 < n; ++c) {
            const int64_t m = n - c - 1;
            const int want = (c + 3 < n) ? 1 : 0;  // column c+1 is reduced next
            double* vnext = want ? vcol(c + 1) : vcol(c);  // (unused when nothing is reduced next)
            step_kernel<<<1, kHouseThreads, 0, s>>>(W, n, c, vcol(c), p, wv, vnext, tau, d, e);
            RT_TRY(check_launch("step_kernel"));
            update_symv_kernel<<<(unsigned)ceil_div((m - 1) * 32, 256), 256, 0, s>>>(W, n, c, vcol(c), wv, vnext,
                                                                                      tau, p, want);
            RT_TRY(check_launch("update_symv_kernel"));
        }
    }
    // d, e of the trailing 2 x 2 (or smaller) block, read on the host with the rest.
    std::vector<double> dh(n), eh(std::max<int64_t>(n, 1), 0.0), tail(4, 0.0);
    RT_CUDA_TRY(cudaMemcpyAsync(dh.data(), d, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s));
    RT_CUDA_TRY(cudaMemcpyAsync(eh.data(), e, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, s));
    const int64_t t0 = std::max<int64_t>(0, n - 2);
    RT_CUDA_TRY(cudaMemcpyAsync(tail.data(), W + t0 * n + t0, sizeof(double) * (size_t)std::min<int64_t>(n, 2),
                                cudaMemcpyDeviceToHost, s));
    if (n >= 2)
        RT_CUDA_TRY(cudaMemcpyAsync(tail.data() + 2, W + (t0 + 1) * n + t0, sizeof(double) * 2,
                                    cudaMemcpyDeviceToHost, s));
    // Q = H_0 H_1 ... H_{n-3}, accumulated backwards.
    identity_kernel<<<g1, 256, 0, s>>>(Q, n);
    RT_TRY(check_launch("identity_kernel"));
    for (int64_t c = n - 3; c >= 0; --c) {
        form_q_kernel<<<(unsigned)ceil_div((n - c - 1) * 32, 256), 256, 0, s>>>(Q, Vst, n, c, tau);
        RT_TRY(check_launch("form_q_kernel"));
    }
    RT_CUDA_TRY(cudaStreamSynchronize(s));
    if (n == 1) {
        dh[0] = tail[0];
    } else {
        dh[n - 2] = tail[0];
        eh[n - 2] = tail[1];
        dh[n - 1] = tail[3];
    }
    Sweeps sw;
    if (!tridiag_qr((int)n, dh, eh, sw)) {
        set_error(RT_ERR_NOT_CONVERGED, "symeig: the tridiagonal QR iteration did not converge (n = %lld)",
                  (long long)n);
        return RT_ERR_NOT_CONVERGED;
    }
    const int nsw = (int)sw.lo.size();
    if (nsw > 0) {
        ScratchBuf rb;
        const size_t ib = align_up(sizeof(int) * (size_t)nsw, 256);
        const size_t fb = align_up(sizeof(int64_t) * (size_t)nsw, 256);
        RT_TRY(scratch_alloc(rb, 2 * ib + fb + sizeof(double2) * sw.rot.size(), s));
        uint8_t* base = rb.as<uint8_t>();
        int* dlo = reinterpret_cast<int*>(base);
        int* dhi = reinterpret_cast<int*>(base + ib);
        int64_t* dfirst = reinterpret_cast<int64_t*>(base + 2 * ib);
        double2* drot = reinterpret_cast<double2*>(base + 2 * ib + fb);
        RT_CUDA_TRY(cudaMemcpyAsync(dlo, sw.lo.data(), sizeof(int) * nsw, cudaMemcpyHostToDevice, s));
        RT_CUDA_TRY(cudaMemcpyAsync(dhi, sw.hi.data(), sizeof(int) * nsw, cudaMemcpyHostToDevice, s));
        RT_CUDA_TRY(cudaMemcpyAsync(dfirst, sw.first.data(), sizeof(int64_t) * nsw, cudaMemcpyHostToDevice, s));
        RT_CUDA_TRY(cudaMemcpyAsync(drot, sw.rot.data(), sizeof(double2) * sw.rot.size(), cudaMemcpyHostToDevice, s));
        // Passes of 32 sweeps, one systolic launch each.
        for (int s0 = 0; s0 < nsw; s0 += 32) {
            rot_systolic_kernel<<<(unsigned)ceil_div(n, kSysRows), kSysRows * 32, 0, s>>>(
                Q, n, dlo, dhi, dfirst, drot, s0, std::min(32, nsw - s0));
            RT_TRY(check_launch("rot_systolic_kernel"));
        }
        RT_CUDA_TRY(cudaStreamSynchronize(s));  // the host vectors above go out of scope
    }
    std::vector<int> perm(n);
    std::iota(perm.begin(), perm.end(), 0);
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) { return dh[a] < dh[b]; });
    std::vector<double> ws(n);
    for (int64_t j = 0; j < n; ++j) ws[j] = dh[perm[j]];
    ScratchBuf pb;
    RT_TRY(scratch_alloc(pb, sizeof(int) * (size_t)n, s));
    RT_CUDA_TRY(cudaMemcpyAsync(pb.p, perm.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, s));
    RT_CUDA_TRY(cudaMemcpyAsync(w, ws.data(), sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, s));
    sort_sign_kernel<<<(unsigned)ceil_div(n * 32, 256), 256, 0, s>>>(Q, V, n, pb.as<int>());
    RT_TRY(check_launch("sort_sign_kernel"));
    RT_CUDA_TRY(cudaStreamSynchronize(s));
    return RT_OK;
}

}  // namespace rt

namespace rt {
namespace {

// V[:, j] *= f[j] for j < ncols.
__global__ void scale_columns_kernel(double* __restrict__ V, int64_t n, int64_t ncols, const double* __restrict__ f) {
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * ncols;
         idx += (int64_t)gridDim.x * blockDim.x)
        V[idx] *= f[idx / n];
}

// Full symmetric A[n, n] from packed upper storage: (i, j), i <= j, at ap[i + j (j + 1) / 2]
// (MatrixUpper, LAPACK 'U' packing).
__global__ void unpack_upper_kernel(const double* __restrict__ ap, double* __restrict__ A, int64_t n) {
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n * n;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = idx % n, j = idx / n;
        const int64_t lo = i < j ? i : j, hi = i < j ? j : i;
        A[idx] = ap[lo + hi * (hi + 1) / 2];
    }
}

unsigned grid_for(int64_t elems) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(elems, 256), 8 * sm_count())); }

// C[m, n] = op(A) op(B) in the float64 or the split form (column-major, leading
// dimensions lda, ldb, m).
rt_status gemm_form(char opa, char opb, int64_t m, int64_t n, int64_t k, const double* A, int64_t lda, const double* B,
                    int64_t ldb, double* C, int form, int nslices, cudaStream_t s) {
    if (form == RT_FORM_SPLIT)
        return rt_dgemm_split(opa, opb, (int)m, (int)n, (int)k, A, (int)lda, B, (int)ldb, C, (int)m, nslices, s);
    GemmF64 g;
    g.opa = opa; g.opb = opb; g.m = m; g.n = n; g.k = k;
    g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.C = C; g.rsC = 1; g.csC = m;
    return gemm_f64(g, s);
}

bool form_ok(int form, int nslices) {
    return form == RT_FORM_FP64 || (form == RT_FORM_SPLIT && nslices >= 3 && nslices <= 8);
}

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" {

rt_status rt_dsyev(int n, double* A, double* w, void* stream) {
    NvtxRange nvtx_range("rt_dsyev");
    RT_REQUIRE(n >= 0, "rt_dsyev: negative order");
    if (n == 0) return RT_OK;
    RT_REQUIRE(A && w, "rt_dsyev: null pointer");
    return symeig_device(n, A, w, A, (cudaStream_t)stream);
}

rt_status rt_lapack_power(const double* S, int n, double p, double threshold, double* out, int* n_nonsingular,
                          int form, int nslices, void* stream) {
    NvtxRange nvtx_range("rt_lapack_power");
    RT_REQUIRE(n >= 0, "rt_lapack_power: negative order");
    RT_REQUIRE(form_ok(form, nslices), "rt_lapack_power: bad form/nslices (%d, %d)", form, nslices);
    if (n_nonsingular) *n_nonsingular = 0;
    if (n == 0) return RT_OK;
    RT_REQUIRE(S && out, "rt_lapack_power: null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    ScratchBuf vb, wb;
    RT_TRY(scratch_alloc(vb, sizeof(double) * (size_t)n * n, s));
    RT_TRY(scratch_alloc(wb, sizeof(double) * (size_t)n, s));
    RT_TRY(symeig_device(n, S, wb.as<double>(), vb.as<double>(), s));
    std::vector<double> w(n), f(n);
    RT_CUDA_TRY(cudaMemcpyAsync(w.data(), wb.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    RT_CUDA_TRY(cudaStreamSynchronize(s));
    // Eigenpairs with eigenvalue >= threshold keep sqrt(ev)^p on their column, the
    // others are dropped (matrix_blas_lapack.rs:1013-1052).
    int kept = 0;
    for (int i = 0; i < n; ++i) {
        if (w[i] >= threshold) {
            f[i] = pow(sqrt(w[i]), p);
            ++kept;
        } else {
            f[i] = 0.0;
        }
    }
    if (n_nonsingular) *n_nonsingular = kept;
    RT_CUDA_TRY(cudaMemcpyAsync(wb.p, f.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    scale_columns_kernel<<<grid_for((int64_t)n * n), 256, 0, s>>>(vb.as<double>(), n, n, wb.as<double>());
    RT_TRY(check_launch("scale_columns_kernel"));
    RT_TRY(gemm_form('N', 'T', n, n, n, vb.as<double>(), n, vb.as<double>(), n, out, form, nslices, s));
    RT_CUDA_TRY(cudaStreamSynchronize(s));  // f leaves scope
    return RT_OK;
}

rt_status rt_dspgvx(const double* ap, const double* bp, int n, int num_orb, double* eigvec, double* w, int form,
                    int nslices, void* stream) {
    NvtxRange nvtx_range("rt_dspgvx");
    RT_REQUIRE(n >= 0, "rt_dspgvx: negative order");
    RT_REQUIRE(form_ok(form, nslices), "rt_dspgvx: bad form/nslices (%d, %d)", form, nslices);
    if (n == 0) return RT_OK;
    RT_REQUIRE(num_orb >= 1 && num_orb <= n, "rt_dspgvx: num_orb = %d must lie in 1..%d", num_orb, n);
    RT_REQUIRE(ap && bp && eigvec && w, "rt_dspgvx: null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nn = (size_t)n * n;
    ScratchBuf fa, fb, ub, tb, vb;
    RT_TRY(scratch_alloc(fa, sizeof(double) * nn, s));
    RT_TRY(scratch_alloc(fb, sizeof(double) * nn, s));
    RT_TRY(scratch_alloc(ub, sizeof(double) * nn, s));
    RT_TRY(scratch_alloc(tb, sizeof(double) * nn, s));
    RT_TRY(scratch_alloc(vb, sizeof(double) * 2 * (size_t)n, s));
    double* Af = fa.as<double>();
    double* Bf = fb.as<double>();
    double* U = ub.as<double>();
    double* T = tb.as<double>();
    double* beta = vb.as<double>();
    double* lam = beta + n;
    unpack_upper_kernel<<<grid_for((int64_t)nn), 256, 0, s>>>(ap, Af, n);
    RT_TRY(check_launch("unpack_upper_kernel"));
    unpack_upper_kernel<<<grid_for((int64_t)nn), 256, 0, s>>>(bp, Bf, n);
    RT_TRY(check_launch("unpack_upper_kernel"));
    // B = U diag(beta) U^T, X = U diag(beta)^-1/2: X^T B X = I.
    RT_TRY(symeig_device(n, Bf, beta, U, s));
    std::vector<double> bh(n);
    RT_CUDA_TRY(cudaMemcpyAsync(bh.data(), beta, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    RT_CUDA_TRY(cudaStreamSynchronize(s));
    if (!(bh[0] > 0.0)) {
        set_error(RT_ERR_INVALID_ARG, "rt_dspgvx: the overlap matrix is not positive definite (smallest eigenvalue %g)",
                  bh[0]);
        return RT_ERR_INVALID_ARG;
    }
    for (int i = 0; i < n; ++i) bh[i] = 1.0 / sqrt(bh[i]);
    RT_CUDA_TRY(cudaMemcpyAsync(beta, bh.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    scale_columns_kernel<<<grid_for((int64_t)nn), 256, 0, s>>>(U, n, n, beta);
    RT_TRY(check_launch("scale_columns_kernel"));
    // C = X^T A X; its eigenvectors Y give x = X y, normalised so that x^T B x = 1.
    RT_TRY(gemm_form('N', 'N', n, n, n, Af, n, U, n, T, form, nslices, s));
    RT_TRY(gemm_form('T', 'N', n, n, n, U, n, T, n, Bf, form, nslices, s));
    RT_TRY(symeig_device(n, Bf, lam, Af, s));
    RT_TRY(gemm_form('N', 'N', n, num_orb, n, U, n, Af, n, eigvec, form, nslices, s));
    // w: the num_orb eigenvalues, then zeros, as dspgvx with range 'I' leaves the reference's vector.
    RT_CUDA_TRY(cudaMemsetAsync(w, 0, sizeof(double) * n, s));
    RT_CUDA_TRY(cudaMemcpyAsync(w, lam, sizeof(double) * num_orb, cudaMemcpyDeviceToDevice, s));
    RT_CUDA_TRY(cudaStreamSynchronize(s));
    return RT_OK;
}

}  // extern "C"
