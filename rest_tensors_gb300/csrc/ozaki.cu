// ozaki.cu - split-precision float64 GEMM on the tcgen05 tensor cores.
//
// Method (error-free splitting, Ozaki et al., "Error-free transformations of
// matrix multiplication by using fast routines of matrix multiplication and
// its applications", Numer. Algorithms 59, 2012; tensor-core variants by
// Mukunoki et al., ISC 2020):
//
//  * Every row of A (and of B, both stored "K-contiguous": C = A B^T) gets a
//    power-of-two scale from its largest exponent.  Each element is turned,
//    with integer operations only, into S signed base-128 digits d_0..d_{S-1}
//    (|d| <= 65, rounded to nearest-even at the last digit):
//        x ~= 2^(e_row - 1028) * sum_s d_s 2^(-7 s)
//    Small integers are exact in BF16, so each digit plane is a BF16 matrix.
//  * Digit planes are multiplied pairwise on tcgen05 (kind::f16, BF16 in,
//    FP32 accumulate in tensor memory).  Products of pairs with the same
//    s + t = g share one TMEM accumulator G_g.  Every partial sum is an
//    integer below 2^24 in magnitude as long as the contraction is cut into
//    chunks of at most floor((2^24 - 1) / (S * 65^2)) terms, so the FP32
//    accumulation is exact.  Pairs with s + t > S - 1 are dropped
//    (their weight is below the last digit's).
//  * The epilogue converts each G_g to an integer, forms
//        V = sum_g G_g 2^(7 (S - 1 - g) - R)
//    in int64 (R, a right shift with round-half-even, keeps V in range over
//    the chunks one CTA accumulates; split-K partials are summed in 128 bits),
//    and rounds once to float64:
//        C = V * 2^(eA + eB - 2056 - 7 (S - 1) + R).
//
// GB300 runs float64 arithmetic at ~1.2 TFLOP/s, so everything above is
// integer or FP32/BF16 work; the only float64 operations are one int64 ->
// float64 conversion per output element.
//
// Data layout.  Digit planes are written by the slicing kernels directly in
// the tensor core's shared-memory operand layout (K-major, no swizzle, 8x16B
// core matrices), pre-tiled as [tile][k-block][digit][T rows x 32 k], so one
// pipeline stage is a handful of 1-D bulk copies (cp.async.bulk) per operand.
#include <algorithm>
#include <cmath>
#include <vector>

#include "rt_internal.cuh"
#include "rt_ptx.cuh"

namespace rt {
namespace oz {

constexpr int TM = 128;        // rows of A per tile (UMMA M)
constexpr int TN = 64;         // rows of B per tile (UMMA N)
constexpr int KB = 16;         // k elements per pipeline stage (one MMA k-step)
constexpr int SK = 32;         // k elements one slicing CTA covers (two k-blocks)
// warp 0 producer, warp 1 MMA, warps 2.. epilogue (16 warps; 8 in the fused form)
constexpr int epi_warps(bool fused) { return fused ? 8 : 16; }
constexpr int NTHREADS = 64 + 32 * epi_warps(false);
constexpr int EPI_THREADS = 256;  // fused form
// Fused variant: warps 10..13 turn float64 tiles staged in shared memory into
// the A digit planes.
constexpr int NTHREADS_FUSED = 448;
constexpr int CONV_THREADS = 128;
constexpr int F64_STAGE = TM * KB * 8;  // float64 staging per pipeline stage
constexpr int kSmemBudget = 220 * 1024;

__host__ __device__ constexpr int stage_bytes(int S, bool fused = false) {
    return S * (TM + TN) * KB * 2 + (fused ? F64_STAGE : 0);
}
__host__ __device__ constexpr int num_stages(int S, bool fused = false) {
    return kSmemBudget / stage_bytes(S, fused) > 6 ? 6 : kSmemBudget / stage_bytes(S, fused);
}
__host__ __device__ constexpr int tmem_cols(int S) { return S * TN <= 256 ? 256 : 512; }

// Accumulator groups.  The product of A digit s and B digit t (s + t <= S-1)
// carries weight 2^(-7(s+t)) and accumulates in group g = s + t, TMEM columns
// [g TN, (g+1) TN).  The MMAs for A digit s stack B digits t0 .. t0+nt-1 (nt <= 4)
// along N; when (S - s) % 4 == 1 the last of them holds B digit S-1-s alone, a
// product of the last group.  Where the allocation has a column block to spare
// (S = 3, 5, 6, 7), those lone products with s >= 1 accumulate there instead,
// in an extra group of the same weight as group S-1 (s = 0's MMAs must cover
// every regular group: they start each chunk by overwriting them).  The widest
// group then has fewer pairs, so an exact chunk is longer.
__host__ __device__ constexpr bool extra_group(int S) { return (S + 1) * TN <= tmem_cols(S); }
__host__ __device__ constexpr bool extra_pair(int S, int s) { return extra_group(S) && s >= 1 && (S - s) % 4 == 1; }
// The MMA warp issues A digit s = issue_digit(S, si) at position si: 0, S-1, 1, S-2, ...
__host__ __device__ constexpr int issue_digit(int S, int si) { return (si & 1) ? S - 1 - (si >> 1) : (si >> 1); }
// The first A digit, in issue order, whose lone product goes to the extra group.
__host__ __device__ constexpr int first_issued_extra_pair(int S) {
    int f = -1;
    for (int si = S - 1; si >= 0; --si) f = extra_pair(S, issue_digit(S, si)) ? issue_digit(S, si) : f;
    return f;
}
// Largest |product| of digits s and t: |d_0| <= 65, |d_s| <= 64 for s >= 1.
__host__ __device__ constexpr int pair_bound(int s, int t) { return (s == 0 ? 65 : 64) * (t == 0 ? 65 : 64); }
// Largest |sum over one k| of group g's products (g == S: the extra group).
__host__ __device__ constexpr int group_bound(int S, int g) {
    int b = 0;
    for (int s = 0; s < S; ++s) {
        const bool moved = extra_pair(S, s);
        if (g == S ? moved : (g - s >= 0 && g - s < S && !(g == S - 1 && moved)))
            b += pair_bound(s, g == S ? S - 1 - s : g - s);
    }
    return b;
}
__host__ __device__ constexpr int max_group_bound(int S) {
    int m = 0;
    for (int g = 0; g <= S; ++g) m = group_bound(S, g) > m ? group_bound(S, g) : m;
    return m;
}
// Longest contraction chunk whose group sums stay exact in FP32 (below 2^24),
// in k-blocks.
__host__ __device__ constexpr int chunk_kblocks(int S) { return ((1 << 24) - 1) / max_group_bound(S) / KB; }
// Groups g and g+1 combine as 128 v_g + v_{g+1} in 32 bits, and group S-1
// with the extra group as v_{S-1} + v_extra, when that cannot overflow over a
// whole chunk.
__host__ __device__ constexpr bool drain_fits_i32(int S) {
    const double n = chunk_kblocks(S) * KB;
    bool ok = true;
    for (int g = 0; g + 1 < S; g += 2)
        ok = ok && 128.0 * group_bound(S, g) * n + (double)group_bound(S, g + 1) * n < 2147483647.0;
    return ok && ((double)group_bound(S, S - 1) + group_bound(S, S)) * n < 2147483647.0;
}
// Balanced chunking: the fewest exact chunks, of near-equal length.
inline int64_t balanced_chunk_kb(int64_t Kb, int S) {
    const int64_t n = ceil_div(Kb, chunk_kblocks(S));
    return ceil_div(Kb, std::max<int64_t>(n, 1));
}
// Byte offset of element (r, k) inside one [T x 16] operand block: 8-row x
// 16-byte core matrices, k-adjacent ones 128 B apart (LBO), row groups 256 B
// apart (SBO).
constexpr uint32_t kLBO = 128, kSBO = 256;
__host__ __device__ __forceinline__ uint32_t core_offset(int r, int k) {
    return (uint32_t)((r & 7) * 16 + (k & 7) * 2 + (k >> 3) * kLBO + (r >> 3) * kSBO);
}

struct Operand {
    const double* p;
    int64_t rows, div, s0, s1, sk;  // elem(r, k) = p[(r % div) * s0 + (r / div) * s1 + k * sk]
};

struct SliceArgs {
    Operand src;
    int64_t K;
    int T;          // tile height (128 for A, 64 for B)
    int64_t tiles;  // ceil(rows / T)
    int64_t Kb;     // ceil(K / 16)
    uint16_t* out;  // [tiles][Kb][S][T*16]
    const int* emax;
    unsigned int* err;
};

// ---------------------------------------------------------------- digits --

template <int S>
struct DigitConst {
    // With t = R + off2, where R is the element in units of the last digit,
    // digit k >= 1 is the 7-bit field at bit 7 (S-1-k), offset by 64; digit 0 is
    // t >> 7 (S-1).  L is the last digit's bit position when the row maximum's
    // leading bit sits at bit 61.
    static constexpr int L = 56 - 7 * (S - 1);
    static constexpr unsigned long long off2() {
        unsigned long long o = 0;
        for (int k = 1; k < S; ++k) o += 64ull << (7 * (S - 1 - k));
        return o;
    }
};

// -------------------------------------------------------------- row scale --

// Biased exponent maximum of each row whose k elements are contiguous (sk == 1):
// one warp per row.
__global__ void emax_contig_kernel(Operand a, int64_t K, int* __restrict__ emax, unsigned int* err) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t r = warp; r < a.rows; r += nwarps) {
        const double* row = a.p + (r % a.div) * a.s0 + (r / a.div) * a.s1;
        unsigned int m = 0;
        for (int64_t k = lane; k < K; k += 32) {
            const unsigned int e = ((unsigned int)__double2hiint(row[k]) >> 20) & 0x7FFu;
            m = max(m, e);
        }
        m = __reduce_max_sync(0xffffffffu, m);
        if (lane == 0) {
            if (m == 0x7FFu) atomicOr(err, DEV_ERR_NONFINITE);
            emax[r] = (int)m;
        }
    }
}

// Same for rows whose consecutive r are contiguous (s0 == 1): thread per row,
// blockIdx.y splits k; results combine through atomicMax on a zeroed array.
__device__ __forceinline__ void emax_strided_body(const Operand& a, int64_t K, int64_t kspan, int* __restrict__ emax,
                                                  unsigned int* err, int64_t bx, int64_t by) {
    const int64_t r = bx * blockDim.x + threadIdx.x;
    if (r >= a.rows) return;
    const int64_t k0 = by * kspan, k1 = min(K, k0 + kspan);
    const double* base = a.p + (r % a.div) * a.s0 + (r / a.div) * a.s1;
    unsigned int m = 0;  // maximum of the sign-cleared high words
    const double* src = base + k0 * a.sk;
    for (int64_t k = k0; k < k1; ++k, src += a.sk) m = max(m, (unsigned int)__double2hiint(*src) & 0x7FFFFFFFu);
    m >>= 20;
    if (m == 0x7FFu) atomicOr(err, DEV_ERR_NONFINITE);
    if (m) atomicMax(&emax[r], (int)m);
}
__global__ void emax_strided_kernel(Operand a, int64_t K, int64_t kspan, int* __restrict__ emax,
                                    unsigned int* err) {
    emax_strided_body(a, K, kspan, emax, err, blockIdx.x, blockIdx.y);
}

// --------------------------------------------------------------- slicing --

// Signed base-128 digits of x relative to the row exponent emax (biased), as
// exact floats:  x ~= 2^(emax - 1028) * sum_s d_s 2^(-7 s),  |d_0| <= 65, |d_s| <= 64.
// The element is rounded once, to nearest with ties to even, at the last
// digit's unit: with m the 53-bit mantissa, that unit is bit P = emax - e + L - 9
// of m, so R = RNE(m / 2^P).  (Ties are common when x is itself the output of
// this GEMM, whose results lie on a coarse power-of-two grid; rounding ties
// away from zero would bias |x| upward.)  Each digit then costs three
// operations: a funnel shift brings its 7-bit field (digit + 64) to the low
// bits, one LOP3 masks it and inserts the exponent of 2^23 (the float 2^23 + u),
// and one FMA by +-1 removes 2^23 + 64 and applies x's sign.
template <int S>
__device__ __forceinline__ void split_digits_f(double x, int emax, float (&f)[S]) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((bits >> 52) & 0x7FF);
    constexpr int L = DigitConst<S>::L;
    const int P = emax - e + L - 9;
    if (e == 0 || P >= 54) {  // zero, subnormal, or below half a unit of the last digit
#pragma unroll
        for (int s = 0; s < S; ++s) f[s] = 0.0f;
        return;
    }
    const unsigned long long m = (bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
    unsigned long long R;
    if (L - 9 <= 0 && P <= 0) R = m << (-P);  // S = 8 only: the grid is finer than the mantissa
    else R = (m + ((1ull << (P - 1)) - 1ull) + ((m >> P) & 1ull)) >> P;
    const unsigned long long t = R + DigitConst<S>::off2();
    const uint32_t hi = (uint32_t)(t >> 32), lo = (uint32_t)t;
    const float sg = (bits >> 63) ? -1.0f : 1.0f;
    constexpr int p0 = 7 * (S - 1);
    const uint32_t w0 = p0 >= 32 ? (hi >> (p0 - 32)) : __funnelshift_r(lo, hi, p0);
    f[0] = __fmaf_rn(__uint_as_float(w0 | 0x4B000000u), sg, -8388608.0f * sg);
    const float c = -8388672.0f * sg;  // -(2^23 + 64) * sign
#pragma unroll
    for (int s = 1; s < S; ++s) {
        const int pos = 7 * (S - 1 - s);
        const uint32_t win = pos >= 32 ? (hi >> (pos - 32)) : __funnelshift_r(lo, hi, pos);
        f[s] = __fmaf_rn(__uint_as_float((win & 127u) | 0x4B000000u), sg, c);
    }
}

// Pack the S digit planes of 8 consecutive k of one row into 16-byte words.
template <int S>
__device__ __forceinline__ void digits8(const double (&x)[8], int em, uint32_t (&w)[S][4]) {
#pragma unroll
    for (int jp = 0; jp < 4; ++jp) {
        float f0[S], f1[S];
        split_digits_f<S>(x[2 * jp], em, f0);
        split_digits_f<S>(x[2 * jp + 1], em, f1);
        // BF16 patterns are the floats' upper halves (the digits have <= 8 significant bits)
#pragma unroll
        for (int s = 0; s < S; ++s) w[s][jp] = __byte_perm(__float_as_uint(f0[s]), __float_as_uint(f1[s]), 0x7632u);
    }
}

template <int S>
__device__ __forceinline__ void store8(const SliceArgs& a, int64_t tile, int64_t kb, int r, int kk,
                                       const uint32_t (&w)[S][4]) {
    uint8_t* blk = reinterpret_cast<uint8_t*>(a.out + ((tile * a.Kb + kb) * S) * (int64_t)(a.T * KB));
#pragma unroll
    for (int s = 0; s < S; ++s)
        *reinterpret_cast<uint4*>(blk + (int64_t)s * a.T * KB * 2 + core_offset(r, kk)) =
            make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
}

// Strided rows (s0 == 1): CTA = (tile, 32 k); work item = (row, 8 consecutive
// k), rows fastest, so reads are coalesced across consecutive rows.
template <int S>
__device__ __forceinline__ void slice_strided_body(const SliceArgs& a, int64_t tile, int64_t k32) {
    const int T = a.T;
    for (int item = threadIdx.x; item < T * (SK / 8); item += blockDim.x) {
        const int r = item % T, q = item / T;
        const int64_t kb = k32 * (SK / KB) + (q >> 1);
        if (kb >= a.Kb) continue;
        const int64_t row = tile * T + r;
        const bool valid = row < a.src.rows;
        const int em = valid ? a.emax[row] : 0;
        const double* base = valid ? a.src.p + (row % a.src.div) * a.src.s0 + (row / a.src.div) * a.src.s1 : nullptr;
        double x[8];
        const int64_t k0 = k32 * SK + q * 8;
        const double* src = base + k0 * a.src.sk;
        if (valid && k0 + 8 <= a.K) {
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = src[j * a.src.sk];
        } else {
#pragma unroll
            for (int j = 0; j < 8; ++j) x[j] = (valid && k0 + j < a.K) ? src[j * a.src.sk] : 0.0;
        }
        uint32_t w[S][4];
        digits8<S>(x, em, w);
        store8<S>(a, tile, kb, r, (q & 1) * 8, w);
    }
}
template <int S>
__global__ void __launch_bounds__(256) slice_strided_kernel(SliceArgs a) {
    slice_strided_body<S>(a, blockIdx.x, blockIdx.y);
}

// Strided rows (s0 == 1) with a short contraction (K <= 8 * (256 / RR) * NBLK):
// row exponents and digits in one pass.  A CTA covers RR rows and all of k;
// thread t takes row t % RR and k-groups t / RR + (256 / RR) j of 8 consecutive
// k, kept in registers.  The threads of a row reduce its exponent maximum
// (shuffles inside a warp, then 8 shared words), then every thread slices its
// runs.  Replaces emax_strided_kernel + slice_strided_kernel (one read of the
// operand instead of two); rows beyond the operand (tile padding) get zero digits.
constexpr int kFusedRows = 16;    // contiguous-row slicer
constexpr int kStridedRows = 16;  // strided-row slicer (8 rows at 3 CTAs/SM measured slower)
constexpr int kStridedRowsWide = 8;  // 640 < K <= 1280: 8 rows, 32 k-groups of 8 per row
constexpr int kStridedRowsShort = 32;  // grouped, K <= 320: 32 rows, 8 k-groups of 8 per row
template <int S, int NBLK, int RR>
__device__ __forceinline__ void slice_strided_rowmax_body(const SliceArgs& a, int* __restrict__ emax_out,
                                                          int64_t blk) {
    constexpr int KQN = 256 / RR;
    __shared__ unsigned int red[8][RR];
    const int r = threadIdx.x % RR;
    const int kq = threadIdx.x / RR;
    const int64_t row = blk * RR + r;
    const bool valid = row < a.src.rows;
    const double* base = valid ? a.src.p + (row % a.src.div) * a.src.s0 + (row / a.src.div) * a.src.s1 : nullptr;
    double x[NBLK][8];
    // Maximum of the sign-cleared high words: its exponent field is the row's.
    unsigned int m = 0;
    const int64_t sk = a.src.sk;
#pragma unroll
    for (int j = 0; j < NBLK; ++j) {
        const int64_t k0 = (int64_t)(kq + KQN * j) * 8;
        const double* src = base + k0 * sk;
        if (valid && k0 + 8 <= a.K) {  // whole run inside k: no per-element tests
#pragma unroll
            for (int i = 0; i < 8; ++i) x[j][i] = src[i * sk];
        } else {
#pragma unroll
            for (int i = 0; i < 8; ++i) x[j][i] = (valid && k0 + i < a.K) ? src[i * sk] : 0.0;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) m = max(m, (unsigned int)__double2hiint(x[j][i]) & 0x7FFFFFFFu);
    }
    m >>= 20;
    // lanes r, r + RR, ... of a warp share the row; then across the 8 warps
#pragma unroll
    for (int o = RR; o < 32; o <<= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) < RR) red[threadIdx.x >> 5][r] = m;
    __syncthreads();
#pragma unroll
    for (int w = 0; w < 8; ++w) m = max(m, red[w][r]);
    if (valid && kq == 0) {
        if (m == 0x7FFu) atomicOr(a.err, DEV_ERR_NONFINITE);
        emax_out[row] = (int)m;
    }
    const int64_t tile = row / a.T;
    const int rt_ = (int)(row % a.T);
#pragma unroll
    for (int j = 0; j < NBLK; ++j) {
        const int64_t k0 = (int64_t)(kq + KQN * j) * 8;
        if (k0 >= a.Kb * KB) continue;
        uint32_t w[S][4];
        digits8<S>(x[j], (int)m, w);
        store8<S>(a, tile, k0 / KB, rt_, (int)(k0 & (KB - 1)), w);
    }
}

template <int S, int NBLK, int RR>
__global__ void __launch_bounds__(256, (RR >= 16 || NBLK > 3) ? 2 : 3)
    slice_strided_rowmax_kernel(SliceArgs a, int* __restrict__ emax_out) {
    slice_strided_rowmax_body<S, NBLK, RR>(a, emax_out, blockIdx.x);
}

// Contiguous rows (sk == 1) with a short contraction (K <= 128 * NBLK): row
// exponents and digits in one pass.  A CTA covers 16 rows.  Warp w handles rows
// 8 (w & 1) .. + 7 (lane & 7) and k-groups 4 (w >> 1) + (lane >> 3); each thread
// keeps NBLK runs of 8 consecutive k (64 contiguous bytes) in registers.  The 16
// threads of a row (4 lanes x 4 warps) reduce its exponent maximum; then every
// thread slices its runs.  Stores of one instruction cover 8 rows x 16 bytes.
template <int S, int NBLK>
__device__ __forceinline__ void slice_contig_rowmax_body(const SliceArgs& a, int* __restrict__ emax_out,
                                                         int64_t blk) {
    __shared__ unsigned int red[4][kFusedRows];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = 8 * (warp & 1) + (lane & 7);
    const int kq = 4 * (warp >> 1) + (lane >> 3);  // 0..15
    const int64_t row = blk * kFusedRows + r;
    const bool valid = row < a.src.rows;
    const double* base = valid ? a.src.p + (row % a.src.div) * a.src.s0 + (row / a.src.div) * a.src.s1 : nullptr;
    double x[NBLK][8];
    unsigned int m = 0;  // maximum of the sign-cleared high words
#pragma unroll
    for (int j = 0; j < NBLK; ++j) {
        const int64_t k0 = (int64_t)(kq + 16 * j) * 8;
        if (valid && k0 + 8 <= a.K) {
#pragma unroll
            for (int i = 0; i < 8; ++i) x[j][i] = base[k0 + i];
        } else {
#pragma unroll
            for (int i = 0; i < 8; ++i) x[j][i] = (valid && k0 + i < a.K) ? base[k0 + i] : 0.0;
        }
#pragma unroll
        for (int i = 0; i < 8; ++i) m = max(m, (unsigned int)__double2hiint(x[j][i]) & 0x7FFFFFFFu);
    }
    m >>= 20;
    // lanes r, r+8, r+16, r+24 share the row within a warp; then 4 warps
    m = max(m, __shfl_xor_sync(0xffffffffu, m, 8));
    m = max(m, __shfl_xor_sync(0xffffffffu, m, 16));
    if (lane < 8) red[warp >> 1][r] = m;
    __syncthreads();
#pragma unroll
    for (int w = 0; w < 4; ++w) m = max(m, red[w][r]);
    if (valid && kq == 0) {
        if (m == 0x7FFu) atomicOr(a.err, DEV_ERR_NONFINITE);
        emax_out[row] = (int)m;
    }
    const int64_t tile = row / a.T;
    const int rt_ = (int)(row % a.T);
#pragma unroll
    for (int j = 0; j < NBLK; ++j) {
        const int64_t k0 = (int64_t)(kq + 16 * j) * 8;
        if (k0 >= a.Kb * KB) continue;
        uint32_t w[S][4];
        digits8<S>(x[j], (int)m, w);
        store8<S>(a, tile, k0 / KB, rt_, (int)(k0 & (KB - 1)), w);
    }
}

template <int S, int NBLK>
__global__ void __launch_bounds__(256, 2) slice_contig_rowmax_kernel(SliceArgs a, int* __restrict__ emax_out) {
    slice_contig_rowmax_body<S, NBLK>(a, emax_out, blockIdx.x);
}

// One-pass slicing of many operands in one launch (the batched products): block
// b belongs to job p with prefix[p] <= b < prefix[p + 1] and runs that job's
// block b - prefix[p].
constexpr int kMaxSliceGroup = 48;
struct SliceGroup {
    SliceArgs a[kMaxSliceGroup];
    int* emax[kMaxSliceGroup];
    int64_t prefix[kMaxSliceGroup + 1];
    int count;
};

__device__ __forceinline__ int slice_job(const SliceGroup& G, int64_t b) {
    int p = 0;
    while (p + 1 < G.count && b >= G.prefix[p + 1]) ++p;
    return p;
}

template <int S, int NBLK, int RR>
__global__ void __launch_bounds__(256, RR >= 16 ? 2 : 3)
    slice_strided_rowmax_grouped(const __grid_constant__ SliceGroup G) {
    const int p = slice_job(G, blockIdx.x);
    slice_strided_rowmax_body<S, NBLK, RR>(G.a[p], G.emax[p], (int64_t)blockIdx.x - G.prefix[p]);
}

template <int S, int NBLK>
__global__ void __launch_bounds__(256, 2) slice_contig_rowmax_grouped(const __grid_constant__ SliceGroup G) {
    const int p = slice_job(G, blockIdx.x);
    slice_contig_rowmax_body<S, NBLK>(G.a[p], G.emax[p], (int64_t)blockIdx.x - G.prefix[p]);
}

// Long contractions over strided rows, two passes for many operands at once:
// job p's blocks are its 2-D grid flattened, x fastest.
constexpr int64_t kStridedSpan = 512;  // k per row-exponent block
__global__ void __launch_bounds__(256) emax_strided_grouped(const __grid_constant__ SliceGroup G) {
    const int p = slice_job(G, blockIdx.x);
    const SliceArgs& a = G.a[p];
    const int64_t b = (int64_t)blockIdx.x - G.prefix[p], gx = (a.src.rows + 255) / 256;
    emax_strided_body(a.src, a.K, kStridedSpan, G.emax[p], a.err, b % gx, b / gx);
}
template <int S>
__global__ void __launch_bounds__(256) slice_strided_grouped(const __grid_constant__ SliceGroup G) {
    const int p = slice_job(G, blockIdx.x);
    const SliceArgs& a = G.a[p];
    const int64_t b = (int64_t)blockIdx.x - G.prefix[p];
    slice_strided_body<S>(a, b % a.tiles, b / a.tiles);
}

// Contiguous rows (sk == 1): the [T x 32] tile is staged through shared
// memory with coalesced row reads, then sliced as above.
template <int S>
__global__ void __launch_bounds__(256) slice_contig_kernel(SliceArgs a) {
    __shared__ double tileb[TM][SK + 1];
    const int T = a.T;
    const int64_t tile = blockIdx.x;
    const int64_t k32 = blockIdx.y;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int rr = wid; rr < T; rr += blockDim.x / 32) {
        const int64_t row = tile * T + rr;
        const int64_t k = k32 * SK + lane;
        double x = 0.0;
        if (row < a.src.rows && k < a.K) x = a.src.p[(row % a.src.div) * a.src.s0 + (row / a.src.div) * a.src.s1 + k];
        tileb[rr][lane] = x;
    }
    __syncthreads();
    for (int item = threadIdx.x; item < T * (SK / 8); item += blockDim.x) {
        const int r = item % T, q = item / T;
        const int64_t kb = k32 * (SK / KB) + (q >> 1);
        if (kb >= a.Kb) continue;
        const int64_t row = tile * T + r;
        const int em = row < a.src.rows ? a.emax[row] : 0;
        double x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = tileb[r][q * 8 + j];
        uint32_t w[S][4];
        digits8<S>(x, em, w);
        store8<S>(a, tile, kb, r, (q & 1) * 8, w);
    }
}

// ------------------------------------------------------------------ GEMM --

struct OutMap {
    double* p;
    int64_t md, ms0, ms1, nd, ns0, ns1;  // addr(m, n) = (m%md)*ms0 + (m/md)*ms1 + (n%nd)*ns0 + (n/nd)*ns1
};

struct GemmArgs {
    const uint8_t* a_slices;  // [tiles_m][Kb][S][TM*KB] bf16
    const uint8_t* b_slices;
    int64_t b_tile2_stride, b_half_stride, b_kb_stride, b_s_stride;  // bytes; 64-row tile tn -> (tn>>1, tn&1)
    int64_t a_kb_stride, a_s_stride, a_tile_stride;                  // bytes
    const int* ea;
    const int* eb;
    int64_t M, N, Kb;
    int64_t tiles_m, tiles_n;
    int chunk_kb;        // k-blocks per exact chunk
    int chunks_per_split;
    int64_t nchunks;     // total chunks
    int R;               // right shift applied to every group (overflow guard)
    int symmetric;       // skip tiles strictly below the diagonal
    OutMap out;
    int64_t* partial;    // splits > 1: [split][tiles_m*TM][tiles_n*TN]
    int splits;
    unsigned int* err;
    // Fused A: float64 source, element (m, k) at a_f64[(m % a_div) + (m / a_div) * a_s1 + k * a_sk].
    const double* a_f64;
    int64_t a_div, a_s1, a_sk, K;
};

__device__ __forceinline__ double scale_pow2(int64_t v, int ex) {
    if (v == 0) return 0.0;
    double r = __ll2double_rn(v);
    const int hi = __double2hiint(r), lo = __double2loint(r);
    const int be = (hi >> 20) & 0x7FF;
    const int ne = be + ex;
    if (ne >= 1 && ne <= 2046) return __hiloint2double(hi + (ex << 20), lo);
    return ldexp(r, ex);
}

// ------------------------------------------------- accumulator drain --
// Group g of a chunk holds, per column, the exact integer sum v_g (in FP32) of
// its digit-pair products; it enters the int64 result as v_g * 2^sh_g with
// sh_g = 7 (S-1-g) - R.  Negative shifts (the overflow guard R) round to
// nearest, ties to even.

// d = a * b + c with a 32 x 32 -> 64-bit signed product.
__device__ __forceinline__ int64_t mad_wide(int32_t a, int32_t b, int64_t c) {
    int64_t d;
    asm("mad.wide.s32 %0, %1, %2, %3;" : "=l"(d) : "r"(a), "r"(b), "l"(c));
    return d;
}

// acc[j] += p(j) * 2^sh for 32-bit integers p(j) and a shift 0 <= sh <= 62 that
// is the same for every j: one multiply-add below 2^31, the high word alone
// from 2^32 up (the low word of p * 2^sh is zero there).
template <int HC, class P>
__device__ __forceinline__ void add_shifted(int64_t (&acc)[HC], int sh, P p) {
    if (sh <= 30) {
        const int32_t mul = 1 << sh;
#pragma unroll
        for (int j = 0; j < HC; ++j) acc[j] = mad_wide(p(j), mul, acc[j]);
    } else if (sh >= 32) {
#pragma unroll
        for (int j = 0; j < HC; ++j) acc[j] += (int64_t)((uint64_t)((uint32_t)p(j) << (sh - 32)) << 32);
    } else {
#pragma unroll
        for (int j = 0; j < HC; ++j) acc[j] += (int64_t)p(j) << sh;
    }
}

// acc[j] += v(j) * 2^sh for 32-bit integers v(j); negative shifts round to
// nearest, ties to even.
template <int HC, class P>
__device__ __forceinline__ void add_value(int64_t (&acc)[HC], int sh, P v) {
    if (sh >= 0) {
        add_shifted<HC>(acc, sh, v);
    } else {
        const int s = -sh;
        const int64_t half = (1ll << (s - 1)) - 1;
#pragma unroll
        for (int j = 0; j < HC; ++j) {
            const int64_t w = (int64_t)v(j);
            acc[j] += (w + half + ((w >> s) & 1)) >> s;
        }
    }
}

__device__ __forceinline__ int32_t f2i(uint32_t bits) { return __float2int_rn(__uint_as_float(bits)); }

// One group, with shift sh.
template <int HC>
__device__ __forceinline__ void add_group(int64_t (&acc)[HC], const uint32_t (&r)[HC], int sh) {
    add_value<HC>(acc, sh, [&](int j) { return f2i(r[j]); });
}

// Two groups of the same weight (group S-1 and the extra group), with shift sh.
template <int HC>
__device__ __forceinline__ void add_group_sum(int64_t (&acc)[HC], const uint32_t (&x)[HC], const uint32_t (&y)[HC],
                                              int sh) {
    add_value<HC>(acc, sh, [&](int j) { return f2i(x[j]) + f2i(y[j]); });
}

// Groups g and g+1 (g+1 < S).  Where group g+1's shift sh is not negative,
// (v_g << (sh+7)) + (v_{g+1} << sh) is formed as (128 v_g + v_{g+1}) << sh with
// the bracket in 32 bits, which the chunk length keeps exact (drain_fits_i32).
template <int S, int HC>
__device__ __forceinline__ void add_group_pair(int64_t (&acc)[HC], const uint32_t (&x)[HC], const uint32_t (&y)[HC],
                                               int g, int R) {
    const int sh = 7 * (S - 2 - g) - R;
    if (sh >= 0) {
        add_shifted<HC>(acc, sh, [&](int j) { return f2i(x[j]) * 128 + f2i(y[j]); });
    } else {
        add_group<HC>(acc, x, sh + 7);
        add_group<HC>(acc, y, sh);
    }
}

// This thread's lane of HC consecutive TMEM columns.
__device__ __forceinline__ void tmem_ld_cols(uint32_t taddr, uint32_t (&r)[16]) { ptx::tmem_ld16(taddr, r); }
__device__ __forceinline__ void tmem_ld_cols(uint32_t taddr, uint32_t (&r)[32]) { ptx::tmem_ld32(taddr, r); }

__device__ __forceinline__ int64_t out_addr(const OutMap& o, int64_t m, int64_t n) {
    return (m % o.md) * o.ms0 + (m / o.md) * o.ms1 + (n % o.nd) * o.ns0 + (n / o.nd) * o.ns1;
}

// First column tile of row tile tm that reaches the diagonal (symmetric products
// compute only tiles with tn * TN + TN - 1 >= tm * TM).
__host__ __device__ __forceinline__ int64_t sym_first_tn(int64_t tm) {
    const int64_t lo = tm * TM - TN + 1;
    return lo > 0 ? (lo + TN - 1) / TN : 0;
}

// Work item w of the persistent grid: tile (tm, tn) and split z; false if the
// item has nothing to do (an empty chunk range).  A symmetric product lists only
// its tiles on or above the diagonal, row by row, so every item carries work and
// consecutive CTAs get equal shares.
__device__ __forceinline__ bool work_item(const GemmArgs& a, int64_t w, int64_t& tm, int64_t& tn, int64_t& c0,
                                          int64_t& c1, int& z) {
    int64_t tile = w / a.splits;
    z = (int)(w % a.splits);
    if (a.symmetric) {
        tm = 0;
        for (;;) {
            const int64_t first = sym_first_tn(tm);
            const int64_t cnt = a.tiles_n > first ? a.tiles_n - first : 0;
            if (tile < cnt || tm + 1 >= a.tiles_m) {
                tn = first + tile;
                break;
            }
            tile -= cnt;
            ++tm;
        }
        if (tn >= a.tiles_n) return false;
    } else {
        tn = tile % a.tiles_n;
        tm = tile / a.tiles_n;
    }
    c0 = (int64_t)z * a.chunks_per_split;
    c1 = min(a.nchunks, c0 + a.chunks_per_split);
    return c0 < c1;
}

// Several independent products in one launch: their work lists are
// concatenated (prefix[p] = first work item of problem p).  Passed by value, so
// a launch captured in a CUDA graph carries its own copy.
template <int MAXG>
struct GroupArgs {
    int n;
    int64_t prefix[MAXG + 1];
    GemmArgs a[MAXG];
};
constexpr int kMaxGroup = 48;

// Persistent split-precision GEMM: one CTA per SM walks the work list with
// stride gridDim.x.  Producer and MMA run ahead across tile boundaries; the
// epilogue hands the tensor memory back as soon as it has read a chunk, so
// the next chunk's MMAs overlap the previous tile's conversion and stores.
template <int S, bool FUSED, int MAXG>
__global__ void __launch_bounds__(FUSED ? NTHREADS_FUSED : NTHREADS, 1)
    oz_gemm_kernel(const __grid_constant__ GroupArgs<MAXG> G) {
    constexpr int STAGES = num_stages(S, FUSED);
    constexpr uint32_t A_BLK = TM * KB * 2;  // one digit plane, bytes
    constexpr uint32_t B_BLK = TN * KB * 2;
    constexpr uint32_t A_STAGE = S * A_BLK;
    constexpr uint32_t DIGITS = S * (A_BLK + B_BLK);
    constexpr uint32_t STAGE = stage_bytes(S, FUSED);  // digits, then (fused) float64 staging
    constexpr uint32_t NCOLS = tmem_cols(S);

    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE);
    uint64_t* empty = full + STAGES;
    uint64_t* f64_full = empty + STAGES;   // fused: float64 tile landed
    uint64_t* f64_empty = f64_full + STAGES;  // fused: converters finished reading it
    uint64_t* acc_full = f64_empty + STAGES;
    uint64_t* acc_empty = acc_full + 1;
    uint64_t* drain = acc_empty + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nitems = G.prefix[G.n];
    unsigned int* const err = G.a[0].err;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            // Fused: the A digits are written by the converter threads, the B
            // digits by a bulk copy announced with arrive.expect_tx.
            ptx::mbar_init(&full[s], FUSED ? CONV_THREADS + 1 : 1);
            ptx::mbar_init(&empty[s], 1);
            ptx::mbar_init(&f64_full[s], 1);
            ptx::mbar_init(&f64_empty[s], CONV_THREADS);
        }
        ptx::mbar_init(acc_full, 1);
        ptx::mbar_init(acc_empty, 32 * epi_warps(FUSED));
        ptx::mbar_init(drain, 1);
        ptx::fence_mbar_init();
    }
    if (warp == 1) {
        ptx::tmem_alloc(tmem_slot, NCOLS);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // ---------------- producer: bulk copies of pre-tiled digit planes
            int64_t it = 0;
            bool ok = true;
            int p = 0;
            for (int64_t w = blockIdx.x; w < nitems && ok; w += gridDim.x) {
                while (w >= G.prefix[p + 1]) ++p;
                const GemmArgs& a = G.a[p];
                int64_t tm, tn, c0, c1;
                int z;
                if (!work_item(a, w - G.prefix[p], tm, tn, c0, c1, z)) continue;
                const uint8_t* abase = a.a_slices + tm * a.a_tile_stride;
                const uint8_t* bbase = a.b_slices + (tn >> 1) * a.b_tile2_stride + (tn & 1) * a.b_half_stride;
                // Fused: the tile's rows m0..m1 split into runs that stay inside one
                // slab (at most 3 for TM = 128 rows); found once per work item.
                int nseg = 0;
                int32_t seg_dst[3] = {0, 0, 0}, seg_len[3] = {0, 0, 0};
                int64_t seg_src[3] = {0, 0, 0};
                const int64_t m0 = tm * TM, m1 = min(a.M, m0 + TM);
                if constexpr (FUSED) {
                    int64_t q = m0 / a.a_div, rem = m0 - q * a.a_div;
                    for (int64_t r = m0; r < m1 && nseg < 3;) {
                        const int64_t re = min(m1, r + (a.a_div - rem));
                        seg_dst[nseg] = (int32_t)(r - m0);
                        seg_len[nseg] = (int32_t)((re - r) * 8);
                        seg_src[nseg] = rem + q * a.a_s1;
                        ++nseg;
                        r = re;
                        ++q;
                        rem = 0;
                    }
                }
                const int64_t kb1 = min(a.Kb, c1 * a.chunk_kb);
                for (int64_t kb = c0 * a.chunk_kb; kb < kb1; ++kb, ++it) {
                    const int st = (int)(it % STAGES);
                    const uint32_t ph = (uint32_t)((it / STAGES) & 1);
                    uint8_t* sa = smem + st * STAGE;
                    uint8_t* sb = sa + A_STAGE;
                    if constexpr (FUSED) {
                        // float64 rows m0..m1 for k-rows k0..k1 into the staging buffer [k][TM].
                        if (!ptx::mbar_wait(&f64_empty[st], ph ^ 1u, a.err)) { ok = false; break; }
                        double* stg = reinterpret_cast<double*>(sa + DIGITS);
                        const int64_t k0 = kb * KB, k1 = min(a.K, k0 + KB);
                        ptx::mbar_arrive_expect_tx(&f64_full[st], (uint32_t)((k1 - k0) * (m1 - m0) * 8));
                        const double* src = a.a_f64 + k0 * a.a_sk;
                        for (int64_t k = k0; k < k1; ++k, src += a.a_sk) {
                            double* dst = stg + (k - k0) * TM;
                            for (int g = 0; g < nseg; ++g)
                                ptx::bulk_g2s(dst + seg_dst[g], src + seg_src[g], (uint32_t)seg_len[g], &f64_full[st]);
                        }
                        if (!ptx::mbar_wait(&empty[st], ph ^ 1u, a.err)) { ok = false; break; }
                        ptx::mbar_arrive_expect_tx(&full[st], S * B_BLK);
                    } else {
                        if (!ptx::mbar_wait(&empty[st], ph ^ 1u, a.err)) { ok = false; break; }
                        ptx::mbar_arrive_expect_tx(&full[st], DIGITS);
                        ptx::bulk_g2s(sa, abase + kb * a.a_kb_stride, A_STAGE, &full[st]);
                    }
                    // B's digit planes of one k-block are contiguous unless B is A's own
                    // 128-row tiles (a product with itself): one copy, else one per plane.
                    if (a.b_s_stride == B_BLK) {
                        ptx::bulk_g2s(sb, bbase + kb * a.b_kb_stride, S * B_BLK, &full[st]);
                    } else {
#pragma unroll
                        for (int s = 0; s < S; ++s)
                            ptx::bulk_g2s(sb + s * B_BLK, bbase + kb * a.b_kb_stride + s * a.b_s_stride, B_BLK,
                                          &full[st]);
                    }
                }
            }
            if (!ok) {
                // Let copies already issued land before the CTA can exit.
                for (int64_t j = max((int64_t)0, it - STAGES); j < it; ++j) {
                    if (FUSED) ptx::mbar_wait(&f64_full[j % STAGES], (uint32_t)((j / STAGES) & 1), err);
                    else ptx::mbar_wait(&full[j % STAGES], (uint32_t)((j / STAGES) & 1), err);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---------------- MMA issuer
            bool ok = true;
            int64_t it = 0, cc = 0;
            const uint32_t sbase = ptx::smem_u32(smem);
            const uint64_t adesc0 = ptx::smem_desc_kmajor_noswizzle(sbase, kLBO, kSBO);
            const uint64_t bdesc0 = ptx::smem_desc_kmajor_noswizzle(sbase + A_STAGE, kLBO, kSBO);
            int p = 0;
            for (int64_t w = blockIdx.x; w < nitems && ok; w += gridDim.x) {
                while (w >= G.prefix[p + 1]) ++p;
                const GemmArgs& a = G.a[p];
                int64_t tm, tn, c0, c1;
                int z;
                if (!work_item(a, w - G.prefix[p], tm, tn, c0, c1, z)) continue;
                for (int64_t c = c0; c < c1 && ok; ++c, ++cc) {
                    if (cc > 0) {
                        if (!ptx::mbar_wait(acc_empty, (uint32_t)((cc - 1) & 1), a.err)) { ok = false; break; }
                        ptx::tc_fence_after();
                    }
                    const int64_t kb1 = min(a.Kb, (c + 1) * (int64_t)a.chunk_kb);
                    bool first = true;
                    for (int64_t kb = c * a.chunk_kb; kb < kb1; ++kb, ++it) {
                        const int st = (int)(it % STAGES);
                        const uint32_t ph = (uint32_t)((it / STAGES) & 1);
                        if (!ptx::mbar_wait(&full[st], ph, a.err)) { ok = false; break; }
                        ptx::tc_fence_after();
                        // Descriptors differ between stages only in the start-address field
                        // (bits 0-13, address >> 4), which never carries for shared memory.
                        const uint64_t soff = (uint64_t)((st * STAGE) >> 4);
                        // For digit s of A, the B digit planes t = 0 .. S-1-s sit back to back in
                        // shared memory and form one K-major operand of 64*(S-s) rows; their
                        // products land in adjacent accumulator groups s .. S-1.  One MMA with
                        // N = 64*(S-s) (split at 256) therefore covers all pairs of digit s.
                        // A digits are issued in the order 0, S-1, 1, S-2, ..., which interleaves
                        // wide and narrow MMAs.  A digit 0 comes first: its MMAs start every
                        // regular group on a chunk's first k-step.  A lone product of the last
                        // group with s >= 1 goes to the extra group (column block S), which the
                        // first of them in issue order starts.
#pragma unroll
                        for (int si = 0; si < S; ++si) {
                            const int s = issue_digit(S, si);
#pragma unroll
                            for (int t0 = 0; t0 < S - s; t0 += 4) {
                                const int nt = (S - s - t0) < 4 ? (S - s - t0) : 4;
                                const bool xg = extra_pair(S, s) && t0 + 1 == S - s;
                                const uint32_t acc = (first && s == (xg ? first_issued_extra_pair(S) : 0)) ? 0u : 1u;
                                ptx::mma_bf16_ss(tmem + (uint32_t)((xg ? S : s + t0) * TN),
                                                 adesc0 + soff + (uint64_t)((s * A_BLK) >> 4),
                                                 bdesc0 + soff + (uint64_t)((t0 * B_BLK) >> 4),
                                                 ptx::idesc_bf16_f32(TM, TN * nt), acc);
                            }
                        }
                        ptx::mma_commit(&empty[st]);
                        first = false;
                    }
                    if (ok) ptx::mma_commit(acc_full);
                }
            }
            // Every MMA issued so far has completed once `drain` fires.
            ptx::mma_commit(drain);
            ptx::mbar_wait(drain, 0, err);
        }
    } else if (FUSED && warp >= 10) {
        // ---------------- converters (fused): float64 staging -> A digit planes
        const int r = threadIdx.x - EPI_THREADS - 64;  // tile row 0..127
        int64_t it = 0;
        bool ok = true;
        int p = 0;
        for (int64_t w = blockIdx.x; w < nitems && ok; w += gridDim.x) {
            while (w >= G.prefix[p + 1]) ++p;
            const GemmArgs& a = G.a[p];
            int64_t tm, tn, c0, c1;
            int z;
            if (!work_item(a, w - G.prefix[p], tm, tn, c0, c1, z)) continue;
            const int64_t m = tm * TM + r;
            const bool valid = m < a.M;
            const int em = valid ? a.ea[m] : 0;
            const int64_t kb1 = min(a.Kb, c1 * a.chunk_kb);
            for (int64_t kb = c0 * a.chunk_kb; kb < kb1; ++kb, ++it) {
                const int st = (int)(it % STAGES);
                const uint32_t ph = (uint32_t)((it / STAGES) & 1);
                uint8_t* sa = smem + st * STAGE;
                const double* stg = reinterpret_cast<const double*>(sa + DIGITS);
                if (!ptx::mbar_wait(&f64_full[st], ph, a.err)) { ok = false; break; }
                const int kv = (int)min((int64_t)KB, a.K - kb * KB);
                double x0[8], x1[8];
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    x0[j] = (valid && j < kv) ? stg[j * TM + r] : 0.0;
                    x1[j] = (valid && j + 8 < kv) ? stg[(j + 8) * TM + r] : 0.0;
                }
                ptx::mbar_arrive(&f64_empty[st]);
                if (!ptx::mbar_wait(&empty[st], ph ^ 1u, a.err)) { ok = false; break; }
                uint32_t w0[S][4], w1[S][4];
                digits8<S>(x0, em, w0);
                digits8<S>(x1, em, w1);
#pragma unroll
                for (int s = 0; s < S; ++s) {
                    *reinterpret_cast<uint4*>(sa + s * A_BLK + core_offset(r, 0)) =
                        make_uint4(w0[s][0], w0[s][1], w0[s][2], w0[s][3]);
                    *reinterpret_cast<uint4*>(sa + s * A_BLK + core_offset(r, 8)) =
                        make_uint4(w1[s][0], w1[s][1], w1[s][2], w1[s][3]);
                }
                ptx::fence_proxy_async_smem();
                ptx::mbar_arrive(&full[st]);
            }
        }
    } else {
        // ---------------- epilogue: warp w reads TMEM lane quadrant w % 4 (its
        // hardware-assigned lanes) and one of epi_warps / 4 column slices.
        constexpr int HC = TN / (epi_warps(FUSED) / 4);
        static_assert(HC % 16 == 0, "column slice must be whole 16-column loads");
        const int q = warp & 3;
        const int h = (warp - 2) >> 2;
        const int rl = 32 * q + lane;
        int64_t cc = 0;
        bool ok = true;
        int p = 0;
        for (int64_t w = blockIdx.x; w < nitems && ok; w += gridDim.x) {
            while (w >= G.prefix[p + 1]) ++p;
            const GemmArgs& a = G.a[p];
            int64_t tm, tn, c0, c1;
            int z;
            if (!work_item(a, w - G.prefix[p], tm, tn, c0, c1, z)) continue;
            const int64_t m = tm * TM + rl;
            int64_t acc[HC];
#pragma unroll
            for (int j = 0; j < HC; ++j) acc[j] = 0;
            for (int64_t c = c0; c < c1; ++c, ++cc) {
                if (!ptx::mbar_wait(acc_full, (uint32_t)(cc & 1), a.err)) { ok = false; break; }
                ptx::tc_fence_after();
                // Groups are read in pairs, one load round each (with 16 columns per
                // thread; one group per round with 32, for registers): (0,1), (2,3), ...,
                // and group S-1 with the extra group.  The tensor memory is handed back
                // to the MMA warp as soon as the last round's loads have landed, before
                // its conversion.
                const uint32_t col = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(h * HC);
                auto release = [&]() {
                    ptx::tc_fence_before();
                    ptx::mbar_arrive(acc_empty);
                };
                const int sh_last = -a.R;  // shift of group S-1 (and of the extra group)
                uint32_t x[HC];
                if constexpr (HC <= 16) {
                    static_assert(drain_fits_i32(S), "paired drain would overflow 32 bits");
                    uint32_t y[HC];
                    // Rounds: pairs (g, g+1) for even g < S-1; then, for odd S, group S-1
                    // (with the extra group); for even S with an extra group, that alone.
                    constexpr int ROUNDS = (S + 1) / 2 + ((S % 2 == 0 && extra_group(S)) ? 1 : 0);
#pragma unroll 1
                    for (int u = 0; u < ROUNDS; ++u) {
                        const int g = 2 * u;
                        const bool last = u + 1 == ROUNDS;
                        if (g + 1 < S) {
                            tmem_ld_cols(col + (uint32_t)(g * TN), x);
                            tmem_ld_cols(col + (uint32_t)((g + 1) * TN), y);
                            ptx::tmem_wait_ld();
                            if (last) release();
                            add_group_pair<S, HC>(acc, x, y, g, a.R);
                        } else if (g == S - 1) {
                            tmem_ld_cols(col + (uint32_t)(g * TN), x);
                            if constexpr (extra_group(S)) tmem_ld_cols(col + (uint32_t)(S * TN), y);
                            ptx::tmem_wait_ld();
                            if (last) release();
                            if constexpr (extra_group(S)) add_group_sum<HC>(acc, x, y, sh_last);
                            else add_group<HC>(acc, x, sh_last);
                        } else {
                            tmem_ld_cols(col + (uint32_t)(S * TN), x);
                            ptx::tmem_wait_ld();
                            if (last) release();
                            add_group<HC>(acc, x, sh_last);
                        }
                    }
                } else {
                    constexpr int ROUNDS = S + (extra_group(S) ? 1 : 0);
#pragma unroll 1
                    for (int g = 0; g < ROUNDS; ++g) {
                        tmem_ld_cols(col + (uint32_t)(g * TN), x);
                        ptx::tmem_wait_ld();
                        if (g + 1 == ROUNDS) release();
                        add_group<HC>(acc, x, g < S ? 7 * (S - 1 - g) - a.R : sh_last);
                    }
                }
            }
            if (!ok || m >= a.M) continue;
            const int64_t n0 = tn * TN + h * HC;
            if (a.splits > 1) {
                int64_t* dst = a.partial + ((int64_t)z * a.tiles_m * TM + m) * (a.tiles_n * TN) + n0;
#pragma unroll
                for (int j = 0; j < HC; ++j) dst[j] = acc[j];
            } else {
                const int base_ex = a.ea[m] - 2056 - 7 * (S - 1) + a.R;
#pragma unroll
                for (int j = 0; j < HC; ++j) {
                    const int64_t n = n0 + j;
                    if (n < a.N) a.out.p[out_addr(a.out, m, n)] = scale_pow2(acc[j], base_ex + a.eb[n]);
                }
            }
        }
    }
    ptx::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        ptx::tc_fence_after();
        ptx::tmem_dealloc(tmem, NCOLS);
    }
}

// Correctly rounded float64 of a signed 128-bit integer times 2^ex.
__device__ __forceinline__ double scale_pow2_i128(__int128 v, int ex) {
    if (v == 0) return 0.0;
    const bool neg = v < 0;
    unsigned __int128 a = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
    int s = 0;
    // Bring |v| below 2^63 keeping a sticky bit; 10+ guard bits remain above
    // the 53-bit significand, so the final conversion rounds correctly.
    while ((a >> 63) != 0) {
        const unsigned __int128 lost = a & 1;
        a >>= 1;
        a |= lost;
        ++s;
    }
    const int64_t w = neg ? -(int64_t)a : (int64_t)a;
    return scale_pow2(w, ex + s);
}

// Sum split-K int64 partials exactly in 128 bits and round once to float64.
template <int S>
__device__ __forceinline__ void finalize_elem(const GemmArgs& a, int64_t idx) {
    const int64_t ldp = a.tiles_n * TN;
    const int64_t n = idx / a.M, m = idx % a.M;
    if (a.symmetric && n < m) return;
    __int128 v = 0;
    for (int z = 0; z < a.splits; ++z) v += (__int128)a.partial[((int64_t)z * a.tiles_m * TM + m) * ldp + n];
    const int ex = a.ea[m] + a.eb[n] - 2056 - 7 * (S - 1) + a.R;
    a.out.p[out_addr(a.out, m, n)] = scale_pow2_i128(v, ex);
}
template <int S>
__global__ void oz_finalize_kernel(GemmArgs a) {
    const int64_t total = a.M * a.N;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x)
        finalize_elem<S>(a, idx);
}

// C(m, n) = C(n, m) for m > n (the symmetric product computes n >= m).
__device__ __forceinline__ void mirror_elem(const OutMap& o, int64_t N, int64_t idx) {
    const int64_t m = idx % N, n = idx / N;
    if (m > n) o.p[out_addr(o, m, n)] = o.p[out_addr(o, n, m)];
}
__global__ void mirror_kernel(OutMap o, int64_t N) {
    const int64_t total = N * N;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x)
        mirror_elem(o, N, idx);
}

// The same for many products in one launch: block b does 1024 output elements
// of the product whose range of blocks (prefix) holds b.
constexpr int64_t kFinishBlock = 1024;
template <int S, int MAXG, bool MIRROR>
__global__ void __launch_bounds__(256) finish_grouped(const __grid_constant__ GroupArgs<MAXG> G) {
    int p = 0;
    while (p + 1 < G.n && (int64_t)blockIdx.x >= G.prefix[p + 1]) ++p;
    const GemmArgs& a = G.a[p];
    const int64_t e0 = ((int64_t)blockIdx.x - G.prefix[p]) * kFinishBlock;
    const int64_t e1 = min(e0 + kFinishBlock, a.M * a.N);
    for (int64_t idx = e0 + threadIdx.x; idx < e1; idx += blockDim.x) {
        if (MIRROR) mirror_elem(a.out, a.M, idx);
        else finalize_elem<S>(a, idx);
    }
}

template <int S>
void set_smem_attr() {
    const int plain = num_stages(S, false) * stage_bytes(S, false) + 256;
    const int fused = num_stages(S, true) * stage_bytes(S, true) + 256;
    cudaFuncSetAttribute(oz_gemm_kernel<S, false, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, plain);
    cudaFuncSetAttribute(oz_gemm_kernel<S, true, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, fused);
    cudaFuncSetAttribute(oz_gemm_kernel<S, false, kMaxGroup>, cudaFuncAttributeMaxDynamicSharedMemorySize, plain);
    cudaFuncSetAttribute(oz_gemm_kernel<S, true, kMaxGroup>, cudaFuncAttributeMaxDynamicSharedMemorySize, fused);
}

// The fused path streams A's float64 rows with 1-D bulk copies: every run of
// rows must start 16-byte aligned and have an even length.
// A tile's 128 rows must also fall into at most 3 such runs (runs of at least
// 64 rows), the size of the producer's per-tile run table.
bool can_fuse_a(const OzOperand& A, bool reuse) {
    const bool short_runs = A.div < A.rows;
    return !reuse && A.s0 == 1 && A.sk != 1 && (!short_runs || (A.div % 2 == 0 && A.div >= TM / 2)) &&
           A.s1 % 2 == 0 && A.sk % 2 == 0 && A.rows % 2 == 0 && ((uintptr_t)A.p % 16) == 0 && A.rows >= TM;
}

struct Sliced {
    ScratchBuf planes, emax;  // owned scratch (unused when the planes come from a prepared operand)
    uint16_t* pl = nullptr;   // the digit planes [tiles][Kb][S][T*16]
    int* em = nullptr;        // row exponents
    int64_t tiles = 0, Kb = 0;
    int T = 0;
};

// Per-row biased exponent maxima only (for the fused path, whose digits are
// formed inside the GEMM).
template <int S>
rt_status row_exponents(const Operand& op, int64_t K, int* emax, cudaStream_t stream) {
    unsigned int* err = error_word_device();
    RT_REQUIRE(err != nullptr, "oz: device error word unavailable");
    RT_CUDA_TRY(cudaMemsetAsync(emax, 0, sizeof(int) * (size_t)op.rows, stream));
    const int64_t kspan = 512;
    dim3 g1((unsigned)ceil_div(op.rows, 256), (unsigned)ceil_div(K, kspan));
    emax_strided_kernel<<<g1, 256, 0, stream>>>(op, K, kspan, emax, err);
    return check_launch("emax_strided_kernel");
}

// One-pass slicing jobs collected by the grouped path and launched together.
struct SliceJob {
    int kind;   // 0: contiguous rows, 1: strided rows (16 per CTA), 2 / 3: row exponents / digits of long
                // strided rows, 4: short strided rows (32 per CTA)
    int nblk;   // the kernel's NBLK
    SliceArgs sa;
    int* emax;
    int64_t blocks;
};
struct SliceQueue {
    std::vector<SliceJob> jobs;
};

template <int S>
rt_status launch_slice_group(int kind, int nblk, const SliceGroup& G, unsigned grid, cudaStream_t stream) {
    constexpr int RR = kStridedRows, KQN = 256 / RR;
    if (kind == 2) {
        emax_strided_grouped<<<grid, 256, 0, stream>>>(G);
        return check_launch("emax_strided_grouped");
    }
    if (kind == 3) {
        slice_strided_grouped<S><<<grid, 256, 0, stream>>>(G);
        return check_launch("slice_strided_grouped");
    }
    if (kind == 4) {
        constexpr int RS = kStridedRowsShort;
        switch (nblk) {
            case 1: slice_strided_rowmax_grouped<S, 1, RS><<<grid, 256, 0, stream>>>(G); break;
            case 2: slice_strided_rowmax_grouped<S, 2, RS><<<grid, 256, 0, stream>>>(G); break;
            case 3: slice_strided_rowmax_grouped<S, 3, RS><<<grid, 256, 0, stream>>>(G); break;
            case 4: slice_strided_rowmax_grouped<S, 4, RS><<<grid, 256, 0, stream>>>(G); break;
            default: slice_strided_rowmax_grouped<S, 5, RS><<<grid, 256, 0, stream>>>(G); break;
        }
        return check_launch("slice_strided_rowmax_grouped");
    }
    if (kind == 0) {
        switch (nblk) {
            case 1: slice_contig_rowmax_grouped<S, 1><<<grid, 256, 0, stream>>>(G); break;
            case 2: slice_contig_rowmax_grouped<S, 2><<<grid, 256, 0, stream>>>(G); break;
            case 3: slice_contig_rowmax_grouped<S, 3><<<grid, 256, 0, stream>>>(G); break;
            case 4: slice_contig_rowmax_grouped<S, 4><<<grid, 256, 0, stream>>>(G); break;
            default: slice_contig_rowmax_grouped<S, 5><<<grid, 256, 0, stream>>>(G); break;
        }
        return check_launch("slice_contig_rowmax_grouped");
    }
    switch (nblk) {
        case 1: slice_strided_rowmax_grouped<S, 1, RR><<<grid, 256, 0, stream>>>(G); break;
        case 2: slice_strided_rowmax_grouped<S, 2, RR><<<grid, 256, 0, stream>>>(G); break;
        case 3: slice_strided_rowmax_grouped<S, 3, RR><<<grid, 256, 0, stream>>>(G); break;
        case 4: slice_strided_rowmax_grouped<S, 4, RR><<<grid, 256, 0, stream>>>(G); break;
        default: slice_strided_rowmax_grouped<S, (640 + 8 * KQN - 1) / (8 * KQN), RR><<<grid, 256, 0, stream>>>(G);
            break;
    }
    return check_launch("slice_strided_rowmax_grouped");
}

// Launch the queued jobs: one grouped launch per (kind, NBLK) and per 48 jobs.
// Row exponents of long strided rows (kind 2) all go before their digits (kind 3).
template <int S>
rt_status flush_slices(SliceQueue& q, cudaStream_t stream) {
    std::vector<bool> done(q.jobs.size(), false);
    std::vector<size_t> order;
    for (int pass = 0; pass < 2; ++pass)
        for (size_t i = 0; i < q.jobs.size(); ++i)
            if ((q.jobs[i].kind == 3) == (pass == 1)) order.push_back(i);
    for (size_t i : order) {
        if (done[i]) continue;
        const int kind = q.jobs[i].kind, nblk = q.jobs[i].nblk;
        SliceGroup G{};
        G.count = 0;
        G.prefix[0] = 0;
        for (size_t j = i; j < q.jobs.size(); ++j) {
            if (done[j] || q.jobs[j].kind != kind || q.jobs[j].nblk != nblk) continue;
            G.a[G.count] = q.jobs[j].sa;
            G.emax[G.count] = q.jobs[j].emax;
            G.prefix[G.count + 1] = G.prefix[G.count] + q.jobs[j].blocks;
            ++G.count;
            done[j] = true;
            if (G.count == kMaxSliceGroup) {
                RT_TRY(launch_slice_group<S>(kind, nblk, G, (unsigned)G.prefix[G.count], stream));
                G.count = 0;
            }
        }
        if (G.count > 0) RT_TRY(launch_slice_group<S>(kind, nblk, G, (unsigned)G.prefix[G.count], stream));
    }
    q.jobs.clear();
    return RT_OK;
}

// Digit planes of one operand.  With a queue, the one-pass cases are recorded
// there (their planes allocated now) and launched later by flush_slices.
// Digit-plane bytes of an operand of `rows` rows sliced in tiles of T rows.
inline size_t plane_bytes(int64_t rows, int64_t K, int T, int S) {
    return (size_t)ceil_div(rows, T) * T * (size_t)ceil_div(K, KB) * KB * 2 * S;
}

// With ext_planes / ext_emax the digits go to caller-owned memory of
// plane_bytes(...) and op.rows ints (a prepared operand), else to scratch.
template <int S>
rt_status slice_operand(const Operand& op, int64_t K, int T, Sliced& out, cudaStream_t stream,
                        SliceQueue* queue = nullptr, uint16_t* ext_planes = nullptr, int* ext_emax = nullptr) {
    out.T = T;
    out.tiles = ceil_div(op.rows, T);
    out.Kb = ceil_div(K, KB);
    if (ext_planes) {
        out.pl = ext_planes;
        out.em = ext_emax;
    } else {
        RT_TRY(scratch_alloc(out.planes, plane_bytes(op.rows, K, T, S), stream));
        RT_TRY(scratch_alloc(out.emax, sizeof(int) * (size_t)std::max<int64_t>(op.rows, 1), stream));
        out.pl = out.planes.as<uint16_t>();
        out.em = out.emax.as<int>();
    }
    unsigned int* err = error_word_device();
    RT_REQUIRE(err != nullptr, "oz: device error word unavailable");
    SliceArgs sa{};
    sa.src = op; sa.K = K; sa.T = T; sa.tiles = out.tiles; sa.Kb = out.Kb;
    sa.out = out.pl; sa.emax = out.em; sa.err = err;
    if (op.sk == 1 && out.Kb * KB <= 128 * 5) {
        const unsigned grid = (unsigned)(out.tiles * T / kFusedRows);
        if (queue) {
            queue->jobs.push_back(SliceJob{0, (int)std::min<int64_t>(ceil_div(out.Kb, 8), 5), sa, out.em,
                                           (int64_t)grid});
            return RT_OK;
        }
        switch ((int)ceil_div(out.Kb, 8)) {
            case 1: slice_contig_rowmax_kernel<S, 1><<<grid, 256, 0, stream>>>(sa, out.em); break;
            case 2: slice_contig_rowmax_kernel<S, 2><<<grid, 256, 0, stream>>>(sa, out.em); break;
            case 3: slice_contig_rowmax_kernel<S, 3><<<grid, 256, 0, stream>>>(sa, out.em); break;
            case 4: slice_contig_rowmax_kernel<S, 4><<<grid, 256, 0, stream>>>(sa, out.em); break;
            default: slice_contig_rowmax_kernel<S, 5><<<grid, 256, 0, stream>>>(sa, out.em); break;
        }
        RT_TRY(check_launch("slice_contig_rowmax_kernel"));
    } else if (op.sk == 1) {
        const int64_t warps = std::min<int64_t>(op.rows, 64ll * sm_count());
        emax_contig_kernel<<<(unsigned)ceil_div(warps * 32, 256), 256, 0, stream>>>(op, K, out.em, err);
        RT_TRY(check_launch("emax_contig_kernel"));
        dim3 grid((unsigned)out.tiles, (unsigned)ceil_div(K, SK));
        slice_contig_kernel<S><<<grid, 256, 0, stream>>>(sa);
        RT_TRY(check_launch("slice_contig_kernel"));
    } else if (op.s0 == 1 && out.Kb * KB <= 640) {
        constexpr int RR = kStridedRows, KQN = 256 / RR;
        const unsigned grid = (unsigned)(out.tiles * T / RR);
        if (queue && out.Kb * KB <= 320) {
            // Short rows (small molecules): 32 rows per CTA keep more of its k-slots busy
            // and give each warp 256-byte runs.
            constexpr int RS = kStridedRowsShort, KQS = 256 / RS;
            const int nb = (int)ceil_div(out.Kb * KB, 8 * KQS);
            queue->jobs.push_back(SliceJob{4, nb, sa, out.em, (int64_t)(out.tiles * T / RS)});
            return RT_OK;
        }
        if (queue) {
            const int nb = (int)ceil_div(out.Kb * KB, 8 * KQN);
            queue->jobs.push_back(SliceJob{1, nb <= 4 ? nb : 5, sa, out.em, (int64_t)grid});
            return RT_OK;
        }
        switch ((int)ceil_div(out.Kb * KB, 8 * KQN)) {
            case 1: slice_strided_rowmax_kernel<S, 1, RR><<<grid, 256, 0, stream>>>(sa, out.em); break;
            case 2: slice_strided_rowmax_kernel<S, 2, RR><<<grid, 256, 0, stream>>>(sa, out.em); break;
            case 3: slice_strided_rowmax_kernel<S, 3, RR><<<grid, 256, 0, stream>>>(sa, out.em); break;
            case 4: slice_strided_rowmax_kernel<S, 4, RR><<<grid, 256, 0, stream>>>(sa, out.em); break;
            default: slice_strided_rowmax_kernel<S, (640 + 8 * KQN - 1) / (8 * KQN), RR>
                         <<<grid, 256, 0, stream>>>(sa, out.em); break;
        }
        RT_TRY(check_launch("slice_strided_rowmax_kernel"));
    } else if (op.s0 == 1 && out.Kb * KB <= 1280) {
        // Still one pass: 8 rows per CTA give each row 32 threads, so five
        // register blocks of 8 k cover 1280 terms.
        constexpr int RR = kStridedRowsWide, KQN = 256 / RR;
        const unsigned grid = (unsigned)(out.tiles * T / RR);
        switch ((int)ceil_div(out.Kb * KB, 8 * KQN)) {
            case 3: slice_strided_rowmax_kernel<S, 3, RR><<<grid, 256, 0, stream>>>(sa, out.em); break;
            case 4: slice_strided_rowmax_kernel<S, 4, RR><<<grid, 256, 0, stream>>>(sa, out.em); break;
            default: slice_strided_rowmax_kernel<S, 5, RR><<<grid, 256, 0, stream>>>(sa, out.em); break;
        }
        RT_TRY(check_launch("slice_strided_rowmax_kernel"));
    } else if (op.s0 == 1) {
        RT_CUDA_TRY(cudaMemsetAsync(out.em, 0, sizeof(int) * (size_t)op.rows, stream));
        if (queue) {
            queue->jobs.push_back(SliceJob{2, 0, sa, out.em, ceil_div(op.rows, (int64_t)256) * ceil_div(K, kStridedSpan)});
            queue->jobs.push_back(SliceJob{3, 0, sa, out.em, out.tiles * ceil_div(K, (int64_t)SK)});
            return RT_OK;
        }
        const int64_t kspan = kStridedSpan;
        dim3 g1((unsigned)ceil_div(op.rows, 256), (unsigned)ceil_div(K, kspan));
        emax_strided_kernel<<<g1, 256, 0, stream>>>(op, K, kspan, out.em, err);
        RT_TRY(check_launch("emax_strided_kernel"));
        dim3 grid((unsigned)out.tiles, (unsigned)ceil_div(K, SK));
        slice_strided_kernel<S><<<grid, 256, 0, stream>>>(sa);
        RT_TRY(check_launch("slice_strided_kernel"));
    } else {
        set_error(RT_ERR_UNSUPPORTED, "oz: operand needs unit stride along k or along rows");
        return RT_ERR_UNSUPPORTED;
    }
    return RT_OK;
}

// One product ready to launch: its digit planes (or, fused, A's row
// exponents), split-K partials and kernel arguments.
struct Prepared {
    Sliced sa, sb;
    ScratchBuf part;
    GemmArgs a{};
    bool fused = false;
    int64_t items = 0;    // work items (tiles x splits)
    int64_t active = 0;   // output tiles that carry work (upper triangle when symmetric)
    int chunks_per_item = 0;
    double flops = 0.0;   // algorithmic digit-pair tensor work
    double slice_bytes = 0.0;
};

template <int S>
void ensure_attrs() {
    static bool done = false;
    if (!done) {
        set_smem_attr<S>();
        done = true;
    }
}

// Slicing and argument set-up for one product; the GEMM itself is launched by
// launch_group, possibly together with other products.
template <int S>
rt_status prepare(const OzGemm& g, Prepared& P, cudaStream_t stream, SliceQueue* queue = nullptr) {
    ensure_attrs<S>();
    Operand A{g.A.p, g.A.rows, g.A.div, g.A.s0, g.A.s1, g.A.sk};
    Operand B{g.B.p, g.B.rows, g.B.div, g.B.s0, g.B.s1, g.B.sk};
    Sliced& sa = P.sa;
    Sliced& sb = P.sb;
    const bool reuse = g.b_is_a;
    const bool fused = !g.a_planes && g.allow_fuse && can_fuse_a(g.A, reuse);
    P.fused = fused;
    // Slicing is HBM-bound: count bytes (8 read + 2*S written per element; the
    // fused path only reads A's float64 once for its row exponents).
    const double slice_bytes = g.a_planes ? (reuse ? 0.0 : (double)B.rows * g.K * (8.0 + 2.0 * S))
                               : fused ? (double)A.rows * g.K * 8.0 + (double)B.rows * g.K * (8.0 + 2.0 * S)
                                       : (double)(A.rows + (reuse ? 0 : B.rows)) * (double)g.K * (8.0 + 2.0 * S);
    // With a queue, the caller times the grouped slicing itself.
    if (!queue) prof_begin(PROF_OZ_SLICE, stream);
    if (g.a_planes) {  // A sliced once beforehand (a prepared operand)
        sa.T = TM;
        sa.tiles = ceil_div(A.rows, TM);
        sa.Kb = ceil_div(g.K, KB);
        sa.pl = const_cast<uint16_t*>(g.a_planes);
        sa.em = const_cast<int*>(g.a_emax);
    } else if (fused) {
        sa.T = TM;
        sa.tiles = ceil_div(A.rows, TM);
        sa.Kb = ceil_div(g.K, KB);
        RT_TRY(scratch_alloc(sa.emax, sizeof(int) * (size_t)A.rows, stream));
        sa.em = sa.emax.as<int>();
        RT_TRY(row_exponents<S>(A, g.K, sa.em, stream));
    } else {
        RT_TRY(slice_operand<S>(A, g.K, TM, sa, stream, queue));
    }
    if (!reuse) RT_TRY(slice_operand<S>(B, g.K, TN, sb, stream, queue));
    if (!queue) prof_end(PROF_OZ_SLICE, stream, slice_bytes);
    P.slice_bytes = slice_bytes;

    GemmArgs& a = P.a;
    if (fused) {
        a.a_f64 = A.p;
        a.a_div = A.div;
        a.a_s1 = A.s1;
        a.a_sk = A.sk;
    }
    a.K = g.K;
    a.a_slices = reinterpret_cast<const uint8_t*>(sa.pl);
    a.a_s_stride = TM * KB * 2;
    a.a_kb_stride = (int64_t)S * TM * KB * 2;
    a.a_tile_stride = sa.Kb * a.a_kb_stride;
    if (reuse) {
        a.b_slices = reinterpret_cast<const uint8_t*>(sa.pl);
        a.b_tile2_stride = a.a_tile_stride;
        a.b_half_stride = TN * KB * 2;
        a.b_kb_stride = a.a_kb_stride;
        a.b_s_stride = a.a_s_stride;
        a.eb = sa.em;
    } else {
        a.b_slices = reinterpret_cast<const uint8_t*>(sb.pl);
        a.b_s_stride = TN * KB * 2;
        a.b_kb_stride = (int64_t)S * TN * KB * 2;
        a.b_half_stride = sb.Kb * a.b_kb_stride;
        a.b_tile2_stride = 2 * a.b_half_stride;
        a.eb = sb.em;
    }
    a.ea = sa.em;
    a.M = A.rows;
    a.N = B.rows;
    a.Kb = sa.Kb;
    a.tiles_m = ceil_div(a.M, TM);
    a.tiles_n = ceil_div(a.N, TN);
    a.chunk_kb = (int)balanced_chunk_kb(a.Kb, S);
    a.nchunks = ceil_div(a.Kb, a.chunk_kb);
    a.symmetric = g.symmetric;
    a.out = OutMap{g.C.p, g.C.md, g.C.ms0, g.C.ms1, g.C.nd, g.C.ns0, g.C.ns1};
    a.err = error_word_device();

    int64_t active = a.tiles_m * a.tiles_n;
    if (g.symmetric) {
        active = 0;
        for (int64_t tm = 0; tm < a.tiles_m; ++tm) active += std::max<int64_t>(0, a.tiles_n - sym_first_tn(tm));
    }
    P.active = active;
    P.chunks_per_item = g.chunks_per_item;
    P.flops = 2.0 * (double)a.M * (double)a.N * (double)g.K * (g.symmetric ? 0.5 : 1.0) * S * (S + 1) / 2;
    return RT_OK;
}

// Split-K plan of one prepared product.  group_active is the number of active
// output tiles of every product that shares the launch: the chunk range is
// split across CTAs only when the whole launch has too few tiles to fill the
// GPU, with the split count whose CTA total best fills whole waves.
template <int S>
rt_status plan(Prepared& P, int64_t group_active, cudaStream_t stream) {
    GemmArgs& a = P.a;
    const int64_t tiles = P.active;
    int64_t splits = 1;
    const int64_t sms = sm_count();
    if (group_active < sms && a.nchunks > 1) {
        double best = 0.0;
        for (int64_t w = 1; w <= 4; ++w) {
            const int64_t sp = std::min<int64_t>(a.nchunks, std::max<int64_t>(1, (w * sms) / group_active));
            const double eff = (double)(group_active * sp) / (double)(ceil_div(group_active * sp, sms) * sms);
            if (eff > best + 0.02) { best = eff; splits = sp; }
        }
    }
    if (P.chunks_per_item > 0) splits = ceil_div(a.nchunks, (int64_t)P.chunks_per_item);
    a.chunks_per_split = (int)ceil_div(a.nchunks, splits);
    splits = ceil_div(a.nchunks, a.chunks_per_split);
    a.splits = (int)splits;
    // Overflow guard for the int64 accumulator of one CTA: over n contraction
    // terms, |V| <= n * 65^2 * 2^(7(S-1)-R) * sum_g (g+1) 2^(-7g) < n * 4292 * 2^(7(S-1)-R),
    // kept below 2^62.  Split-K partials are summed in 128 bits, so only the
    // terms one CTA sees count.
    {
        const double terms = (double)a.chunks_per_split * a.chunk_kb * KB;
        const int need = (int)std::ceil(std::log2(terms * 4292.0)) + 7 * (S - 1) - 62;
        a.R = std::max(0, need);
    }
    if (splits > 1) {
        RT_TRY(scratch_alloc(P.part, sizeof(int64_t) * (size_t)splits * a.tiles_m * TM * a.tiles_n * TN, stream));
        a.partial = P.part.as<int64_t>();
    }
    P.items = tiles * splits;
    return RT_OK;
}

// One persistent launch over the work items of n prepared products (all of
// the same fused mode).
template <int S, int MAXG>
rt_status launch_group(Prepared* const* ps, int n, cudaStream_t stream) {
    static_assert(sizeof(GroupArgs<MAXG>) <= 32000, "kernel parameter block too large");
    GroupArgs<MAXG> G;
    G.n = n;
    G.prefix[0] = 0;
    double flops = 0.0;
    for (int i = 0; i < n; ++i) {
        G.a[i] = ps[i]->a;
        G.prefix[i + 1] = G.prefix[i] + ps[i]->items;
        flops += ps[i]->flops;
    }
    for (int i = n; i < MAXG; ++i) G.prefix[i + 1] = G.prefix[n];
    if (G.prefix[n] == 0) return RT_OK;
    const bool fused = ps[0]->fused;
    dim3 grid((unsigned)std::min<int64_t>(G.prefix[n], sm_count()));
    prof_begin(PROF_OZ_GEMM, stream);
    if (fused)
        oz_gemm_kernel<S, true, MAXG>
            <<<grid, NTHREADS_FUSED, num_stages(S, true) * stage_bytes(S, true) + 256, stream>>>(G);
    else
        oz_gemm_kernel<S, false, MAXG>
            <<<grid, NTHREADS, num_stages(S, false) * stage_bytes(S, false) + 256, stream>>>(G);
    prof_end(PROF_OZ_GEMM, stream, flops);
    return check_launch("oz_gemm_kernel");
}

// Split-K reduction and symmetric mirror of one product.
template <int S>
rt_status finish(const Prepared& P, cudaStream_t stream) {
    if (P.a.splits > 1) {
        oz_finalize_kernel<S><<<4 * sm_count(), 256, 0, stream>>>(P.a);
        RT_TRY(check_launch("oz_finalize_kernel"));
    }
    if (P.a.symmetric) {
        mirror_kernel<<<4 * sm_count(), 256, 0, stream>>>(P.a.out, P.a.M);
        RT_TRY(check_launch("mirror_kernel"));
    }
    return RT_OK;
}

template <int S>
rt_status run(const OzGemm& g, cudaStream_t stream) {
    Prepared P;
    RT_TRY(prepare<S>(g, P, stream));
    RT_TRY(plan<S>(P, P.active, stream));
    Prepared* ps[1] = {&P};
    RT_TRY((launch_group<S, 1>(ps, 1, stream)));
    return finish<S>(P, stream);
}

// Split-K reductions, then symmetric mirrors, of many products: one grouped
// launch of each per 48 products.
template <int S>
rt_status finish_many(const std::vector<Prepared>& P, cudaStream_t stream) {
    for (int mirror = 0; mirror < 2; ++mirror) {
        std::vector<const Prepared*> list;
        for (const Prepared& x : P)
            if ((mirror ? x.a.symmetric != 0 : x.a.splits > 1) && x.a.M * x.a.N > 0) list.push_back(&x);
        for (size_t i0 = 0; i0 < list.size(); i0 += kMaxGroup) {
            const int cnt = (int)std::min<size_t>(kMaxGroup, list.size() - i0);
            GroupArgs<kMaxGroup> G;
            G.n = cnt;
            G.prefix[0] = 0;
            for (int i = 0; i < cnt; ++i) {
                G.a[i] = list[i0 + i]->a;
                G.prefix[i + 1] = G.prefix[i] + ceil_div(G.a[i].M * G.a[i].N, kFinishBlock);
            }
            for (int i = cnt; i < kMaxGroup; ++i) G.prefix[i + 1] = G.prefix[cnt];
            const unsigned grid = (unsigned)G.prefix[cnt];
            if (mirror) finish_grouped<S, kMaxGroup, true><<<grid, 256, 0, stream>>>(G);
            else finish_grouped<S, kMaxGroup, false><<<grid, 256, 0, stream>>>(G);
            RT_TRY(check_launch("finish_grouped"));
        }
    }
    return RT_OK;
}

// Many products, grouped into as few launches as possible.
template <int S>
rt_status run_many(const OzGemm* gs, int n, cudaStream_t stream) {
    std::vector<Prepared> P(n);
    int64_t active = 0;
    SliceQueue queue;
    double slice_bytes = 0.0;
    prof_begin(PROF_OZ_SLICE, stream);
    for (int i = 0; i < n; ++i) {
        RT_TRY(prepare<S>(gs[i], P[i], stream, &queue));
        active += P[i].active;
        slice_bytes += P[i].slice_bytes;
    }
    RT_TRY(flush_slices<S>(queue, stream));
    prof_end(PROF_OZ_SLICE, stream, slice_bytes);
    for (int i = 0; i < n; ++i) RT_TRY(plan<S>(P[i], active, stream));
    for (int mode = 0; mode < 2; ++mode) {
        std::vector<Prepared*> grp;
        for (int i = 0; i < n; ++i)
            if ((int)P[i].fused == mode && P[i].items > 0) grp.push_back(&P[i]);
        for (size_t i0 = 0; i0 < grp.size(); i0 += kMaxGroup) {
            const int cnt = (int)std::min<size_t>(kMaxGroup, grp.size() - i0);
            RT_TRY((launch_group<S, kMaxGroup>(grp.data() + i0, cnt, stream)));
        }
    }
    RT_TRY(finish_many<S>(P, stream));
    return RT_OK;
}

}  // namespace oz

rt_status oz_gemm_many(const OzGemm* gs, int n, cudaStream_t stream) {
    if (n <= 0) return RT_OK;
    const int S = gs[0].nslices;
    for (int i = 0; i < n; ++i) {
        RT_REQUIRE(gs[i].nslices == S, "oz_gemm_many: all products need the same slice count");
        RT_REQUIRE(gs[i].A.rows > 0 && gs[i].B.rows > 0 && gs[i].K > 0, "oz_gemm_many: empty product");
        RT_REQUIRE(!gs[i].symmetric || (gs[i].b_is_a && gs[i].A.rows == gs[i].B.rows),
                   "oz_gemm_many: symmetric needs B == A");
    }
    switch (S) {
        case 3: return oz::run_many<3>(gs, n, stream);
        case 4: return oz::run_many<4>(gs, n, stream);
        case 5: return oz::run_many<5>(gs, n, stream);
        case 6: return oz::run_many<6>(gs, n, stream);
        case 7: return oz::run_many<7>(gs, n, stream);
        case 8: return oz::run_many<8>(gs, n, stream);
        default:
            set_error(RT_ERR_INVALID_ARG, "nslices must be in 3..8 (got %d)", S);
            return RT_ERR_INVALID_ARG;
    }
}

size_t oz_plane_bytes(int64_t rows, int64_t K, int nslices) { return oz::plane_bytes(rows, K, oz::TM, nslices); }

// Digit planes and row exponents of A as the A operand of later products
// (OzGemm::a_planes / a_emax), into caller-owned memory.
rt_status oz_slice_into(const OzOperand& A, int64_t K, int nslices, uint16_t* planes, int* emax,
                        cudaStream_t stream) {
    RT_REQUIRE(A.rows > 0 && K > 0 && planes && emax, "oz_slice_into: bad arguments");
    oz::Operand op{A.p, A.rows, A.div, A.s0, A.s1, A.sk};
    oz::Sliced sl;
    switch (nslices) {
        case 3: return oz::slice_operand<3>(op, K, oz::TM, sl, stream, nullptr, planes, emax);
        case 4: return oz::slice_operand<4>(op, K, oz::TM, sl, stream, nullptr, planes, emax);
        case 5: return oz::slice_operand<5>(op, K, oz::TM, sl, stream, nullptr, planes, emax);
        case 6: return oz::slice_operand<6>(op, K, oz::TM, sl, stream, nullptr, planes, emax);
        case 7: return oz::slice_operand<7>(op, K, oz::TM, sl, stream, nullptr, planes, emax);
        case 8: return oz::slice_operand<8>(op, K, oz::TM, sl, stream, nullptr, planes, emax);
        default:
            set_error(RT_ERR_INVALID_ARG, "nslices must be in 3..8 (got %d)", nslices);
            return RT_ERR_INVALID_ARG;
    }
}

rt_status oz_gemm(const OzGemm& g, cudaStream_t stream) {
    RT_REQUIRE(g.A.rows >= 0 && g.B.rows >= 0 && g.K >= 0, "oz_gemm: negative size");
    RT_REQUIRE(!g.symmetric || (g.b_is_a && g.A.rows == g.B.rows), "oz_gemm: symmetric needs B == A");
    if (g.A.rows == 0 || g.B.rows == 0) return RT_OK;
    switch (g.nslices) {
        case 3: return oz::run<3>(g, stream);
        case 4: return oz::run<4>(g, stream);
        case 5: return oz::run<5>(g, stream);
        case 6: return oz::run<6>(g, stream);
        case 7: return oz::run<7>(g, stream);
        case 8: return oz::run<8>(g, stream);
        default:
            set_error(RT_ERR_INVALID_ARG, "nslices must be in 3..8 (got %d)", g.nslices);
            return RT_ERR_INVALID_ARG;
    }
}

}  // namespace rt
