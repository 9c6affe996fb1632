// rt_internal.cuh - shared internals of the GB300 RI-path library.
//
// Status/error plumbing, stream-ordered scratch, the device error word, and
// the two GEMM services (float64 DFMA and split-precision tcgen05).  Everything here is internal; the public C ABI lives in
// include/rest_tensors_gb300.h.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/rest_tensors_gb300.h"

namespace rt {

// Thread-local text of the most recent failure, returned by rt_last_error().
void set_error(rt_status s, const char* fmt, ...);
rt_status last_status();

#define RT_CUDA_TRY(expr)                                                                       \
    do {                                                                                        \
        cudaError_t _e = (expr);                                                                \
        if (_e != cudaSuccess) {                                                                \
            ::rt::set_error(RT_ERR_CUDA, "%s failed: %s (%s:%d)", #expr, cudaGetErrorString(_e), \
                            __FILE__, __LINE__);                                                \
            return RT_ERR_CUDA;                                                                 \
        }                                                                                       \
    } while (0)

#define RT_TRY(expr)                       \
    do {                                   \
        rt_status _s = (expr);             \
        if (_s != RT_OK) return _s;        \
    } while (0)

#define RT_REQUIRE(cond, ...)                                  \
    do {                                                       \
        if (!(cond)) {                                         \
            ::rt::set_error(RT_ERR_INVALID_ARG, __VA_ARGS__);  \
            return RT_ERR_INVALID_ARG;                         \
        }                                                      \
    } while (0)

// Check for a launch error right after a <<<>>> launch (also counts launches).
rt_status check_launch(const char* what);

// Opt-in kernel timing: when enabled, prof_begin/prof_end bracket a launch
// with CUDA events on its stream and attribute `flops` algorithmic
// operations to the kernel kind.
enum ProfKind : int { PROF_OZ_GEMM = 0, PROF_OZ_SLICE = 1, PROF_DGEMM = 2, PROF_RIJ = 3, PROF_NKINDS = 4 };
bool prof_enabled();
void prof_begin(int kind, cudaStream_t s);
void prof_end(int kind, cudaStream_t s, double flops);

// Stream-ordered scratch from the device's default memory pool
// (cudaMallocAsync / cudaFreeAsync on the call's stream), released when the
// holder goes out of scope.  Concurrent calls on different streams each get
// their own blocks.
struct ScratchBuf {
    void* p = nullptr;
    cudaStream_t s = nullptr;
    ScratchBuf() = default;
    ScratchBuf(const ScratchBuf&) = delete;
    ScratchBuf& operator=(const ScratchBuf&) = delete;
    ~ScratchBuf() {
        if (p) cudaFreeAsync(p, s);
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};
rt_status scratch_alloc(ScratchBuf& b, size_t bytes, cudaStream_t stream);

// Device-wide error word written by kernels that find bad input (non-finite
// values, exhausted waits); read back by the launching entry point.
rt_status error_word_reset(cudaStream_t stream);
rt_status error_word_check(cudaStream_t stream, const char* what);
unsigned int* error_word_device();

enum : unsigned int {
    DEV_ERR_NONFINITE = 1u,
    DEV_ERR_TIMEOUT = 2u,
    DEV_ERR_ASYMMETRIC = 4u,  // a symmetric entry's sampled check found B[mu,nu] != B[nu,mu]
};

// RT_CHECK_SYMMETRY=1 in the environment (read once per process): the entries
// whose contract is symmetric slabs sample mirror pairs of their input.
bool symmetry_check_enabled();
// Device-side check of nslab [nb, nb] slabs: every mirror pair of the first,
// 64 sampled pairs of each.
rt_status symmetry_sample(const double* B, int nb, int64_t nslab, cudaStream_t stream);
// The same on host memory, synchronously; RT_ERR_INVALID_ARG on a mismatch.
rt_status symmetry_sample_host(const double* B, int nb, int64_t nslab, const char* what);

int sm_count();

// NVTX range over one entry point (visible in Nsight timelines; no cost without a tool).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }
inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// "No composite index": a divisor larger than any row count.
constexpr int64_t kNoDiv = (int64_t)1 << 62;

// Strided block copy of float64 elements, the primitive under the layout
// utilities:  out[a0 os0 + a1 os1 + a2 os2] = in[a0 is0 + a1 is1 + a2 is2]
// for a_d < n[d].  Source and destination must not overlap.
struct Copy3 {
    int64_t n[3] = {1, 1, 1}, is[3] = {0, 0, 0}, os[3] = {0, 0, 0};
};
rt_status strided_copy3(const double* in, double* out, const Copy3& c, cudaStream_t stream);

// FP64 GEMM service used by every plain-form contraction.  Column-major.
//   C_b(i,j) = alpha * sum_k opA(A_b)(i,k) opB(B_b)(k,j) + beta * C_b(i,j)
//   A_b = A + b*sA, B_b = B + b*sB,
//   C_b(i,j) at C + i*rsC + j*csC + b*bsC   (rsC may differ from 1, e.g. P-fastest outputs)
struct GemmF64 {
    char opa = 'N', opb = 'N';
    int64_t m = 0, n = 0, k = 0;
    double alpha = 1.0, beta = 0.0;
    const double* A = nullptr;
    int64_t lda = 0, sA = 0;
    const double* B = nullptr;
    int64_t ldb = 0, sB = 0;
    double* C = nullptr;
    int64_t rsC = 1, csC = 0, bsC = 0;
    int64_t batch = 1;
    int splitk = 1;  // >1: partial sums in scratch, reduced deterministically
    // Composite row index (rows that are a pair (r % div, r / div)):
    //   A row r at (r % a_div) + (r / a_div) * a_s1 (opa 'N'; times lda for 'T'),
    //   C row r at (r % c_md) * rsC + (r / c_md) * c_ms1.
    int64_t a_div = kNoDiv, a_s1 = 0;
    int64_t c_md = kNoDiv, c_ms1 = 0;
};
rt_status gemm_f64(const GemmF64& g, cudaStream_t stream);
// Several float64 GEMMs in one launch per op pair and tile shape (k == 0 is
// not accepted here); products with splitk > 1 share one reduction launch.
rt_status gemm_f64_many(const GemmF64* gs, int n, cudaStream_t stream);

// Split-precision (BF16 digit planes on tcgen05, exact integer
// recombination) GEMM, written as C(m, n) = sum_k A(m, k) * B(n, k):
//   A(m, k) at A.p[(m % A.div) * A.s0 + (m / A.div) * A.s1 + k * A.sk]   (likewise B)
//   C(m, n) at C.p[(m % md) * ms0 + (m / md) * ms1 + (n % nd) * ns0 + (n / nd) * ns1]
// Each operand needs unit stride along k (sk == 1) or along rows (s0 == 1).
// nslices in [3, 8].  b_is_a reuses A's digit planes for B; symmetric (with
// b_is_a) computes only n >= m and mirrors.
struct OzOperand {
    const double* p = nullptr;
    int64_t rows = 0, div = kNoDiv, s0 = 0, s1 = 0, sk = 1;
};
struct OzOut {
    double* p = nullptr;
    int64_t md = kNoDiv, ms0 = 1, ms1 = 0, nd = kNoDiv, ns0 = 0, ns1 = 0;
};
struct OzGemm {
    int64_t K = 0;
    OzOperand A, B;
    OzOut C;
    int nslices = 6;
    bool b_is_a = false;
    bool symmetric = false;
    // Form A's digits inside the GEMM (no digit-plane scratch for A) when A's
    // layout allows it.  Off by default: separate slicing is faster on GB300;
    // the fused form trades speed for memory.
    bool allow_fuse = false;
    int chunks_per_item = 0;  // >0: exact chunks per work item (split-K granularity); 0: fill whole waves
    // A already sliced by oz_slice_into with the same nslices (A's layout then only sets rows and K).
    const uint16_t* a_planes = nullptr;
    const int* a_emax = nullptr;
};
rt_status oz_gemm(const OzGemm& g, cudaStream_t stream);
// Bytes of the digit planes of an A operand (rows x K, nslices digits), and the slicing into caller memory.
size_t oz_plane_bytes(int64_t rows, int64_t K, int nslices);
rt_status oz_slice_into(const OzOperand& A, int64_t K, int nslices, uint16_t* planes, int* emax, cudaStream_t stream);
// Several independent products with the same slice count: one slicing pass
// each, then as few grouped persistent GEMM launches as possible.
rt_status oz_gemm_many(const OzGemm* gs, int n, cudaStream_t stream);

}  // namespace rt
