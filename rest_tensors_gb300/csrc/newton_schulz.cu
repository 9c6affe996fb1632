// newton_schulz.cu - inverse square root of a symmetric positive matrix by
// Newton-Schulz iteration, the GEMM-only route REST's SCF side uses for
// S^-1/2 and V^-1/2 (src/matrix/matrix_blas_lapack.rs:1710-1932).
//
// The control flow is the reference's, kept on the host: the level-shift
// stages of _newton_schulz_inverse_square_root_v02 (:1710-1778) and, per
// stage, the iteration, convergence test and mixing branches of
// _newton_schulz_inverse_square_root_lf (:1780-1932).  Every matrix stays in
// HBM.  The three n x n products of a step run on the float64 GEMM (DFMA) or
// the split tcgen05 GEMM; the norms are fixed-order device reductions read
// back once per step, because the next branch depends on them.  Elementwise
// updates use explicit round-to-nearest multiplies and adds, so each one
// rounds as the reference's unfused Rust arithmetic does.
#include <math.h>

#include <algorithm>
#include <vector>

#include "rt_internal.cuh"

namespace rt {
namespace {

constexpr int kRedBlocks = 256;

__global__ void __launch_bounds__(256) ns_div_kernel(double* __restrict__ out, const double* __restrict__ in,
                                                     double s, int64_t n2) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = __ddiv_rn(in[i], s);
}

__global__ void __launch_bounds__(256) ns_mul_kernel(double* __restrict__ x, double s, int64_t n2) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = __dmul_rn(x[i], s);
}

// Level shift (matrix_blas_lapack.rs:1789-1795): diagonal elements above the
// threshold gain the shift, the others become zero.
__global__ void ns_shift_diag_kernel(double* __restrict__ m, int n, double threshold, double shift) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double* d = m + (int64_t)i * n + i;
        *d = *d > threshold ? __dadd_rn(*d, shift) : 0.0;
    }
}

// Initial guess (:1807-1816): a * I, with zeros where |diag(matr)| < threshold.
__global__ void ns_init_guess_kernel(double* __restrict__ x, const double* __restrict__ m, int n, double threshold,
                                     double a) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double d = m[(int64_t)i * n + i];
        x[(int64_t)i * n + i] = fabs(d) < threshold ? 0.0 : a;
    }
}

// u = 3 I + w * (-1)  (par_scaled_add, src/matrix/mod.rs:671-684)
__global__ void __launch_bounds__(256) ns_three_minus_kernel(double* __restrict__ u, const double* __restrict__ w,
                                                             int n) {
    const int64_t n2 = (int64_t)n * n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
        const double three = (i % n == i / n) ? 3.0 : 0.0;
        u[i] = __dadd_rn(three, __dmul_rn(w[i], -1.0));
    }
}

// x = mix * from + (1 - mix) * x
__global__ void __launch_bounds__(256) ns_mix_kernel(double* __restrict__ x, const double* __restrict__ from,
                                                     double mix, int64_t n2) {
    const double keep = 1.0 - mix;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = __dadd_rn(__dmul_rn(mix, from[i]), __dmul_rn(keep, x[i]));
}

// (:1885-1890) x /= t twice, then the diagonal *= t.
__global__ void __launch_bounds__(256) ns_big_rescale_kernel(double* __restrict__ x, double t, int n) {
    const int64_t n2 = (int64_t)n * n;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
        double v = __ddiv_rn(__ddiv_rn(x[i], t), t);
        if (i % n == i / n) v = __dmul_rn(v, t);
        x[i] = v;
    }
}

__global__ void ns_set_diag_kernel(double* __restrict__ x, double a, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[(int64_t)i * n + i] = a;
}

// Fixed-order sums: block b adds elements b, b + G*256, ... per thread and
// reduces them by a tree; ns_finish_kernel adds the G partials in order.
// With y: sums (x - y)^2 and y^2; without: x^2.
__global__ void __launch_bounds__(256) ns_sumsq_kernel(const double* __restrict__ x, const double* __restrict__ y,
                                                       int64_t n2, double* __restrict__ partial) {
    __shared__ double s0[256], s1[256];
    double a = 0.0, b = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n2; i += (int64_t)gridDim.x * blockDim.x) {
        if (y) {
            const double d = __dadd_rn(x[i], -y[i]);
            a = __dadd_rn(a, __dmul_rn(d, d));
            b = __dadd_rn(b, __dmul_rn(y[i], y[i]));
        } else {
            a = __dadd_rn(a, __dmul_rn(x[i], x[i]));
        }
    }
    s0[threadIdx.x] = a;
    s1[threadIdx.x] = b;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s0[threadIdx.x] = __dadd_rn(s0[threadIdx.x], s0[threadIdx.x + w]);
            s1[threadIdx.x] = __dadd_rn(s1[threadIdx.x], s1[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = s0[0];
        partial[2 * blockIdx.x + 1] = s1[0];
    }
}

__global__ void ns_finish_kernel(const double* __restrict__ partial, int nblk, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double a = 0.0, b = 0.0;
    for (int i = 0; i < nblk; ++i) {
        a = __dadd_rn(a, partial[2 * i]);
        b = __dadd_rn(b, partial[2 * i + 1]);
    }
    out[0] = a;
    out[1] = b;
}

class NewtonSchulz {
  public:
    NewtonSchulz(int n, int form, int S, cudaStream_t s) : n_(n), n2_((int64_t)n * n), form_(form), S_(S), s_(s) {}

    rt_status init() {
        RT_TRY(scratch_alloc(buf_, sizeof(double) * (size_t)(6 * n2_ + 2 * kRedBlocks + 2), s_));
        double* p = buf_.as<double>();
        matr_ = p; x_ = p + n2_; t_ = p + 2 * n2_; u_ = p + 3 * n2_; nxt_ = p + 4 * n2_; prev_ = p + 5 * n2_;
        partial_ = p + 6 * n2_;
        red_ = partial_ + 2 * kRedBlocks;
        return RT_OK;
    }

    // C = alpha * A B for column-major n x n matrices.
    rt_status mm(double* C, const double* A, const double* B, double alpha) {
        if (form_ == RT_FORM_FP64) {
            GemmF64 g;
            g.opa = 'N'; g.opb = 'N';
            g.m = n_; g.n = n_; g.k = n_; g.alpha = alpha; g.beta = 0.0;
            g.A = A; g.lda = n_; g.B = B; g.ldb = n_; g.C = C; g.rsC = 1; g.csC = n_;
            return gemm_f64(g, s_);
        }
        OzGemm g;
        g.K = n_;
        g.A.p = A; g.A.rows = n_; g.A.s0 = 1; g.A.sk = n_;
        g.B.p = B; g.B.rows = n_; g.B.s0 = n_; g.B.sk = 1;
        g.C.p = C; g.C.ms0 = 1; g.C.ns0 = n_;
        g.nslices = S_;
        RT_TRY(oz_gemm(g, s_));
        if (alpha != 1.0) {
            ns_mul_kernel<<<grid(), 256, 0, s_>>>(C, alpha, n2_);
            RT_TRY(check_launch("ns_mul_kernel"));
        }
        return RT_OK;
    }

    // {sum (x - y)^2, sum y^2}, or {sum x^2, 0} without y, read back to the host.
    rt_status sums(const double* x, const double* y, double out[2]) {
        ns_sumsq_kernel<<<kRedBlocks, 256, 0, s_>>>(x, y, n2_, partial_);
        RT_TRY(check_launch("ns_sumsq_kernel"));
        ns_finish_kernel<<<1, 32, 0, s_>>>(partial_, kRedBlocks, red_);
        RT_TRY(check_launch("ns_finish_kernel"));
        RT_CUDA_TRY(cudaMemcpyAsync(out, red_, 2 * sizeof(double), cudaMemcpyDeviceToHost, s_));
        RT_CUDA_TRY(cudaStreamSynchronize(s_));
        return RT_OK;
    }

    // X_next = 0.5 X (3I - A X X) into nxt_.
    rt_status step() {
        RT_TRY(mm(t_, matr_, x_, 1.0));
        RT_TRY(mm(nxt_, t_, x_, 1.0));
        ns_three_minus_kernel<<<grid(), 256, 0, s_>>>(u_, nxt_, n_);
        RT_TRY(check_launch("ns_three_minus_kernel"));
        return mm(nxt_, x_, u_, 0.5);
    }

    rt_status mix(double* x, const double* from, double m) {
        ns_mix_kernel<<<grid(), 256, 0, s_>>>(x, from, m, n2_);
        return check_launch("ns_mix_kernel");
    }

    rt_status copy(double* dst, const double* src) {
        RT_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * (size_t)n2_, cudaMemcpyDeviceToDevice, s_));
        return RT_OK;
    }

    // _newton_schulz_inverse_square_root_lf on matr_0 (device), with an
    // optional initial guess (device).  The returned iterate (the last X_next)
    // is left in `out`.
    // `evals` receives the number of X_next evaluations (three products each).
    rt_status lf(const double* matr0, const double* guess, double threshold, double mix_parameter,
                 double level_shift, int num_iter, double* out, bool& converged, int& evals) {
        const double num_elems = (double)n2_;
        RT_TRY(copy(matr_, matr0));
        ns_shift_diag_kernel<<<std::max(1, (n_ + 255) / 256), 256, 0, s_>>>(matr_, n_, threshold, level_shift);
        RT_TRY(check_launch("ns_shift_diag_kernel"));
        // trace / n, summed from the first diagonal element on, as the reference's fold
        std::vector<double> diag(n_);
        RT_CUDA_TRY(cudaMemcpy2DAsync(diag.data(), sizeof(double), matr_, sizeof(double) * (n_ + 1), sizeof(double),
                                      n_, cudaMemcpyDeviceToHost, s_));
        RT_CUDA_TRY(cudaStreamSynchronize(s_));
        double trace = 0.0;
        for (double d : diag) trace += d;
        const double trace_1 = trace / (double)n_;
        const double initial_a = 1.0 / sqrt(trace_1);
        if (guess) {
            RT_TRY(copy(x_, guess));
        } else {
            RT_CUDA_TRY(cudaMemsetAsync(x_, 0, sizeof(double) * (size_t)n2_, s_));
            ns_init_guess_kernel<<<std::max(1, (n_ + 255) / 256), 256, 0, s_>>>(x_, matr_, n_, threshold, initial_a);
            RT_TRY(check_launch("ns_init_guess_kernel"));
        }
        double r[2];
        RT_TRY(step());
        evals = 1;
        RT_TRY(sums(x_, nxt_, r));
        double norm = sqrt(r[0]) / num_elems;
        double prev_norm = norm;
        RT_TRY(copy(x_, nxt_));
        converged = norm <= threshold;
        int count_unchanged = 0;
        for (int it = 0; it < num_iter; ++it) {
            RT_TRY(step());
            ++evals;
            RT_TRY(sums(x_, nxt_, r));
            norm = sqrt(r[0]) / num_elems;
            converged = norm <= threshold;
            const double change_norm = norm - prev_norm;
            prev_norm = norm;
            RT_TRY(copy(prev_, x_));
            if (converged) break;
            if (norm <= threshold * 10.0) {
                RT_TRY(mix(x_, nxt_, mix_parameter));
                RT_TRY(mix(x_, prev_, mix_parameter));
                count_unchanged = 0;
            } else if (change_norm > threshold) {
                count_unchanged = 0;
                RT_TRY(mix(x_, nxt_, mix_parameter));
                double q[2];
                RT_TRY(sums(x_, nullptr, q));
                const double tmp = sqrt(q[0]);
                if (tmp >= 100.0) {
                    ns_big_rescale_kernel<<<grid(), 256, 0, s_>>>(x_, tmp, n_);
                    RT_TRY(check_launch("ns_big_rescale_kernel"));
                }
            } else if (fabs(change_norm) <= threshold) {
                if (count_unchanged < 5) {
                    RT_TRY(mix(x_, nxt_, mix_parameter));
                    ++count_unchanged;
                } else {
                    ns_set_diag_kernel<<<std::max(1, (n_ + 255) / 256), 256, 0, s_>>>(x_, initial_a, n_);
                    RT_TRY(check_launch("ns_set_diag_kernel"));
                    count_unchanged = 0;
                }
            } else {
                RT_TRY(copy(x_, nxt_));
                count_unchanged = 0;
            }
        }
        return copy(out, nxt_);
    }

    unsigned grid() const { return (unsigned)std::min<int64_t>((n2_ + 255) / 256, (int64_t)sm_count() * 8); }

    rt_status div(double* out, const double* in, double s) {
        ns_div_kernel<<<grid(), 256, 0, s_>>>(out, in, s, n2_);
        return check_launch("ns_div_kernel");
    }
    rt_status scale(double* x, double s) {
        ns_mul_kernel<<<grid(), 256, 0, s_>>>(x, s, n2_);
        return check_launch("ns_mul_kernel");
    }

  private:
    int n_;
    int64_t n2_;
    int form_, S_;
    cudaStream_t s_;
    ScratchBuf buf_;
    double *matr_ = nullptr, *x_ = nullptr, *t_ = nullptr, *u_ = nullptr, *nxt_ = nullptr, *prev_ = nullptr;
    double *partial_ = nullptr, *red_ = nullptr;
};

}  // namespace
}  // namespace rt

using namespace rt;

extern "C" rt_status rt_newton_schulz_inv_sqrt(const double* S, int n, double threshold, double mix_parameter,
                                               int num_iter, const double* level_shift, int n_level_shift, int form,
                                               int nslices, double* out, int* converged, int* steps,
                                               void* stream) {
    NvtxRange nvtx_range("rt_newton_schulz_inv_sqrt");
    RT_REQUIRE(n >= 1, "rt_newton_schulz_inv_sqrt: n must be positive");
    RT_REQUIRE(num_iter >= 0, "rt_newton_schulz_inv_sqrt: negative iteration count");
    RT_REQUIRE(n_level_shift >= 1 && level_shift,
               "rt_newton_schulz_inv_sqrt: at least one level shift is required");
    RT_REQUIRE(form == RT_FORM_FP64 || (form == RT_FORM_SPLIT && nslices >= 3 && nslices <= 8),
               "rt_newton_schulz_inv_sqrt: bad form/nslices (%d, %d)", form, nslices);
    RT_REQUIRE(S && out, "rt_newton_schulz_inv_sqrt: null pointer");
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t n2 = (int64_t)n * n;
    NewtonSchulz ns(n, form, nslices, s);
    RT_TRY(ns.init());
    ScratchBuf wb;
    RT_TRY(scratch_alloc(wb, sizeof(double) * (size_t)(2 * n2), s));
    double* matr0 = wb.as<double>();
    double* guess = matr0 + n2;
    // 1) normalise by the Frobenius norm (:1721-1729)
    double r[2];
    RT_TRY(ns.sums(S, nullptr, r));
    const double original_norm = sqrt(r[0]);
    RT_REQUIRE(original_norm > 0.0 && isfinite(original_norm),
               "rt_newton_schulz_inv_sqrt: the matrix norm is zero or not finite");
    RT_TRY(ns.div(matr0, S, original_norm));
    // 2) level-shift stages (:1735-1768)
    bool have_guess = false, conv = false;
    int total = 0;
    for (int i = 0; i < n_level_shift; ++i) {
        bool lf_conv = false;
        int it = 0;
        RT_TRY(ns.lf(matr0, have_guess ? guess : nullptr, threshold, mix_parameter, level_shift[i], num_iter, out,
                     lf_conv, it));
        total += it;
        double fine_mix = mix_parameter;
        if (!lf_conv) {
            bool lf2 = lf_conv;
            int cur = 0;
            while (!lf2) {
                fine_mix = fine_mix / 2.0;
                ++cur;
                RT_TRY(ns.lf(matr0, have_guess ? guess : nullptr, threshold, fine_mix, level_shift[i], num_iter, out,
                             lf2, it));
                total += it;
                if (cur > 5) break;
            }
            RT_CUDA_TRY(cudaMemcpyAsync(guess, out, sizeof(double) * (size_t)n2, cudaMemcpyDeviceToDevice, s));
            have_guess = true;
            conv = lf2;
            break;
        }
        conv = lf_conv;
        RT_CUDA_TRY(cudaMemcpyAsync(guess, out, sizeof(double) * (size_t)n2, cudaMemcpyDeviceToDevice, s));
        have_guess = true;
    }
    // 3) undo the normalisation (:1772-1773)
    RT_CUDA_TRY(cudaMemcpyAsync(out, guess, sizeof(double) * (size_t)n2, cudaMemcpyDeviceToDevice, s));
    RT_TRY(ns.scale(out, pow(original_norm, -0.5)));
    RT_CUDA_TRY(cudaStreamSynchronize(s));
    if (converged) *converged = conv ? 1 : 0;
    if (steps) *steps = total;
    return RT_OK;
}
