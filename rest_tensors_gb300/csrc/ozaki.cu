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

#include "rt_internal.cuh"
#include "rt_ptx.cuh"

namespace rt {
namespace oz {

constexpr int TM = 128;        // rows of A per tile (UMMA M)
constexpr int TN = 64;         // rows of B per tile (UMMA N)
constexpr int KB = 16;         // k elements per pipeline stage (one MMA k-step)
constexpr int SK = 32;         // k elements one slicing CTA covers (two k-blocks)
constexpr int NTHREADS = 320;  // warp 0 producer, warp 1 MMA, warps 2..9 epilogue
constexpr int EPI_THREADS = 256;
constexpr int kSmemBudget = 220 * 1024;

__host__ __device__ constexpr int stage_bytes(int S) { return S * (TM + TN) * KB * 2; }
__host__ __device__ constexpr int num_stages(int S) {
    return kSmemBudget / stage_bytes(S) > 6 ? 6 : kSmemBudget / stage_bytes(S);
}
// Longest contraction chunk whose group sums stay exact in FP32, in k-blocks.
__host__ __device__ constexpr int chunk_kblocks(int S) { return (int)(((1 << 24) - 1) / (S * 65 * 65) / KB); }
// Balanced chunking: the fewest exact chunks, of near-equal length.
inline int64_t balanced_chunk_kb(int64_t Kb, int S) {
    const int64_t n = ceil_div(Kb, chunk_kblocks(S));
    return ceil_div(Kb, std::max<int64_t>(n, 1));
}
__host__ __device__ constexpr int tmem_cols(int S) { return S * TN <= 256 ? 256 : 512; }

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
    // q has the row maximum's leading bit at position 61; digit s sits at bit
    // 56 - 7 s, so the last digit's unit is 2^L.
    static constexpr int L = 56 - 7 * (S - 1);
    static constexpr unsigned long long off() {
        unsigned long long o = 0;
        for (int k = 1; k < S; ++k) o += 1ull << (62 - 7 * k);
        return o;
    }
};

// Signed base-128 digits of x relative to the row exponent emax (biased).
// The last digit is rounded to nearest, ties to even; mantissa bits shifted
// out below q are kept as a sticky bit, so only true ties go to even.  (Ties
// are common when x is itself the output of this GEMM, whose results lie on a
// coarse power-of-two grid; rounding ties away from zero would then bias |x|
// upward.)
template <int S>
__device__ __forceinline__ void split_digits(double x, int emax, int (&d)[S]) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int e = (int)((bits >> 52) & 0x7FF);
    const int sh = emax - e + 1;
    if (e == 0 || sh >= 64) {
#pragma unroll
        for (int s = 0; s < S; ++s) d[s] = 0;
        return;
    }
    const unsigned long long full = ((bits & 0xFFFFFFFFFFFFFull) | (1ull << 52)) << 10;
    unsigned long long q = full >> sh;
    q |= (full & ((1ull << sh) - 1ull)) != 0ull ? 1ull : 0ull;
    constexpr int L = DigitConst<S>::L;
    const unsigned long long t = q + ((1ull << (L - 1)) - 1ull) + ((q >> L) & 1ull) + DigitConst<S>::off();
    const bool neg = (bits >> 63) != 0;
    d[0] = (int)(t >> 56);
#pragma unroll
    for (int s = 1; s < S; ++s) d[s] = (int)((t >> (56 - 7 * s)) & 127ull) - 64;
    if (neg) {
#pragma unroll
        for (int s = 0; s < S; ++s) d[s] = -d[s];
    }
}

// Exact BF16 bit pattern of a small integer (|v| <= 256).
__device__ __forceinline__ uint32_t bf16_of_int(int v) {
    return (uint32_t)__float_as_uint((float)v) >> 16;
}

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
__global__ void emax_strided_kernel(Operand a, int64_t K, int64_t kspan, int* __restrict__ emax,
                                    unsigned int* err) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.rows) return;
    const int64_t k0 = (int64_t)blockIdx.y * kspan, k1 = min(K, k0 + kspan);
    const double* base = a.p + (r % a.div) * a.s0 + (r / a.div) * a.s1;
    unsigned int m = 0;
    for (int64_t k = k0; k < k1; ++k) {
        const unsigned int e = ((unsigned int)__double2hiint(base[k * a.sk]) >> 20) & 0x7FFu;
        m = max(m, e);
    }
    if (m == 0x7FFu) atomicOr(err, DEV_ERR_NONFINITE);
    if (m) atomicMax(&emax[r], (int)m);
}

// --------------------------------------------------------------- slicing --

// Pack the S digit planes of 8 consecutive k of one row into 16-byte words.
template <int S>
__device__ __forceinline__ void digits8(const double (&x)[8], int em, uint32_t (&w)[S][4]) {
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        int d[S];
        split_digits<S>(x[j], em, d);
#pragma unroll
        for (int s = 0; s < S; ++s) {
            const uint32_t h = bf16_of_int(d[s]);
            if (j & 1) w[s][j >> 1] |= h << 16;
            else w[s][j >> 1] = h;
        }
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
__global__ void __launch_bounds__(256) slice_strided_kernel(SliceArgs a) {
    const int T = a.T;
    const int64_t tile = blockIdx.x;
    const int64_t k32 = blockIdx.y;
    for (int item = threadIdx.x; item < T * (SK / 8); item += blockDim.x) {
        const int r = item % T, q = item / T;
        const int64_t kb = k32 * (SK / KB) + (q >> 1);
        if (kb >= a.Kb) continue;
        const int64_t row = tile * T + r;
        const bool valid = row < a.src.rows;
        const int em = valid ? a.emax[row] : 0;
        const double* base = valid ? a.src.p + (row % a.src.div) * a.src.s0 + (row / a.src.div) * a.src.s1 : nullptr;
        double x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int64_t k = k32 * SK + q * 8 + j;
            x[j] = (valid && k < a.K) ? base[k * a.src.sk] : 0.0;
        }
        uint32_t w[S][4];
        digits8<S>(x, em, w);
        store8<S>(a, tile, kb, r, (q & 1) * 8, w);
    }
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

__device__ __forceinline__ int64_t out_addr(const OutMap& o, int64_t m, int64_t n) {
    return (m % o.md) * o.ms0 + (m / o.md) * o.ms1 + (n % o.nd) * o.ns0 + (n / o.nd) * o.ns1;
}

// Work item w of the persistent grid: tile (tm, tn) and split z; false if the
// item has nothing to do (below the diagonal of a symmetric product, or an
// empty chunk range).
__device__ __forceinline__ bool work_item(const GemmArgs& a, int64_t w, int64_t& tm, int64_t& tn, int64_t& c0,
                                          int64_t& c1, int& z) {
    const int64_t tile = w / a.splits;
    z = (int)(w % a.splits);
    tn = tile % a.tiles_n;
    tm = tile / a.tiles_n;
    if (a.symmetric && (tn * TN + TN - 1) < tm * TM) return false;
    c0 = (int64_t)z * a.chunks_per_split;
    c1 = min(a.nchunks, c0 + a.chunks_per_split);
    return c0 < c1;
}

// Persistent split-precision GEMM: one CTA per SM walks the work list with
// stride gridDim.x.  Producer and MMA run ahead across tile boundaries; the
// epilogue hands the tensor memory back as soon as it has read a chunk, so
// the next chunk's MMAs overlap the previous tile's conversion and stores.
template <int S>
__global__ void __launch_bounds__(NTHREADS, 1) oz_gemm_kernel(GemmArgs a) {
    constexpr int STAGES = num_stages(S);
    constexpr uint32_t A_BLK = TM * KB * 2;  // one digit plane, bytes
    constexpr uint32_t B_BLK = TN * KB * 2;
    constexpr uint32_t A_STAGE = S * A_BLK;
    constexpr uint32_t STAGE = S * (A_BLK + B_BLK);
    constexpr uint32_t NCOLS = tmem_cols(S);

    extern __shared__ __align__(1024) uint8_t smem[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE);
    uint64_t* empty = full + STAGES;
    uint64_t* acc_full = empty + STAGES;
    uint64_t* acc_empty = acc_full + 1;
    uint64_t* drain = acc_empty + 1;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t nitems = a.tiles_m * a.tiles_n * a.splits;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            ptx::mbar_init(&full[s], 1);
            ptx::mbar_init(&empty[s], 1);
        }
        ptx::mbar_init(acc_full, 1);
        ptx::mbar_init(acc_empty, EPI_THREADS);
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
            for (int64_t w = blockIdx.x; w < nitems && ok; w += gridDim.x) {
                int64_t tm, tn, c0, c1;
                int z;
                if (!work_item(a, w, tm, tn, c0, c1, z)) continue;
                const uint8_t* abase = a.a_slices + tm * a.a_tile_stride;
                const uint8_t* bbase = a.b_slices + (tn >> 1) * a.b_tile2_stride + (tn & 1) * a.b_half_stride;
                const int64_t kb1 = min(a.Kb, c1 * a.chunk_kb);
                for (int64_t kb = c0 * a.chunk_kb; kb < kb1; ++kb, ++it) {
                    const int st = (int)(it % STAGES);
                    const uint32_t ph = (uint32_t)((it / STAGES) & 1);
                    if (!ptx::mbar_wait(&empty[st], ph ^ 1u, a.err)) { ok = false; break; }
                    uint8_t* sa = smem + st * STAGE;
                    uint8_t* sb = sa + A_STAGE;
                    ptx::mbar_arrive_expect_tx(&full[st], STAGE);
                    ptx::bulk_g2s(sa, abase + kb * a.a_kb_stride, A_STAGE, &full[st]);
#pragma unroll
                    for (int s = 0; s < S; ++s)
                        ptx::bulk_g2s(sb + s * B_BLK, bbase + kb * a.b_kb_stride + s * a.b_s_stride, B_BLK, &full[st]);
                }
            }
            if (!ok) {
                // Let copies already issued land before the CTA can exit.
                for (int64_t j = max((int64_t)0, it - STAGES); j < it; ++j)
                    ptx::mbar_wait(&full[j % STAGES], (uint32_t)((j / STAGES) & 1), a.err);
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
            for (int64_t w = blockIdx.x; w < nitems && ok; w += gridDim.x) {
                int64_t tm, tn, c0, c1;
                int z;
                if (!work_item(a, w, tm, tn, c0, c1, z)) continue;
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
#pragma unroll
                        for (int s = 0; s < S; ++s) {
#pragma unroll
                            for (int t0 = 0; t0 < S - s; t0 += 4) {
                                const int nt = (S - s - t0) < 4 ? (S - s - t0) : 4;
                                const uint32_t acc = (first && s == 0) ? 0u : 1u;
                                ptx::mma_bf16_ss(tmem + (uint32_t)((s + t0) * TN), adesc0 + soff + (uint64_t)((s * A_BLK) >> 4),
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
            ptx::mbar_wait(drain, 0, a.err);
        }
    } else {
        // ---------------- epilogue: 8 warps; warp w reads TMEM lane quadrant w % 4
        // (its hardware-assigned lanes) and one half of the 64 columns.
        constexpr int HC = TN / 2;
        const int q = warp & 3;
        const int h = (warp - 2) >> 2;
        const int rl = 32 * q + lane;
        int64_t cc = 0;
        bool ok = true;
        for (int64_t w = blockIdx.x; w < nitems && ok; w += gridDim.x) {
            int64_t tm, tn, c0, c1;
            int z;
            if (!work_item(a, w, tm, tn, c0, c1, z)) continue;
            const int64_t m = tm * TM + rl;
            int64_t acc[HC];
#pragma unroll
            for (int j = 0; j < HC; ++j) acc[j] = 0;
            for (int64_t c = c0; c < c1; ++c, ++cc) {
                if (!ptx::mbar_wait(acc_full, (uint32_t)(cc & 1), a.err)) { ok = false; break; }
                ptx::tc_fence_after();
#pragma unroll 1
                for (int g = 0; g < S; ++g) {
                    const int sh = 7 * (S - 1 - g) - a.R;
                    uint32_t r0[16], r1[16];
                    const uint32_t col = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(g * TN + h * HC);
                    ptx::tmem_ld16(col, r0);
                    ptx::tmem_ld16(col + 16, r1);
                    ptx::tmem_wait_ld();
                    if (sh >= 0) {
#pragma unroll
                        for (int j = 0; j < HC; ++j)
                            acc[j] += (int64_t)__float2int_rn(__uint_as_float(j < 16 ? r0[j] : r1[j - 16])) << sh;
                    } else {
                        // Right shifts round to nearest, ties to even.
                        const int r = -sh;
                        const int64_t half = (1ll << (r - 1)) - 1;
#pragma unroll
                        for (int j = 0; j < HC; ++j) {
                            const int64_t v = (int64_t)__float2int_rn(__uint_as_float(j < 16 ? r0[j] : r1[j - 16]));
                            acc[j] += (v + half + ((v >> r) & 1)) >> r;
                        }
                    }
                }
                ptx::tc_fence_before();
                ptx::mbar_arrive(acc_empty);
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
__global__ void oz_finalize_kernel(GemmArgs a) {
    const int64_t ldp = a.tiles_n * TN;
    const int64_t total = a.M * a.N;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t n = idx / a.M, m = idx % a.M;
        if (a.symmetric && n < m) continue;
        __int128 v = 0;
        for (int z = 0; z < a.splits; ++z) v += (__int128)a.partial[((int64_t)z * a.tiles_m * TM + m) * ldp + n];
        const int ex = a.ea[m] + a.eb[n] - 2056 - 7 * (S - 1) + a.R;
        a.out.p[out_addr(a.out, m, n)] = scale_pow2_i128(v, ex);
    }
}

// C(m, n) = C(n, m) for m > n (the symmetric product computes n >= m).
__global__ void mirror_kernel(OutMap o, int64_t N) {
    const int64_t total = N * N;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t m = idx % N, n = idx / N;
        if (m > n) o.p[out_addr(o, m, n)] = o.p[out_addr(o, n, m)];
    }
}

template <int S>
void set_smem_attr() {
    constexpr int bytes = num_stages(S) * stage_bytes(S) + 256;
    cudaFuncSetAttribute(oz_gemm_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

struct Sliced {
    ScratchBuf planes, emax;
    int64_t tiles = 0, Kb = 0;
    int T = 0;
};

template <int S>
rt_status slice_operand(const Operand& op, int64_t K, int T, Sliced& out, cudaStream_t stream) {
    out.T = T;
    out.tiles = ceil_div(op.rows, T);
    out.Kb = ceil_div(K, KB);
    const size_t plane_bytes = (size_t)out.tiles * T * (size_t)out.Kb * KB * 2 * S;
    RT_TRY(scratch_alloc(out.planes, plane_bytes, stream));
    RT_TRY(scratch_alloc(out.emax, sizeof(int) * (size_t)std::max<int64_t>(op.rows, 1), stream));
    unsigned int* err = error_word_device();
    RT_REQUIRE(err != nullptr, "oz: device error word unavailable");
    SliceArgs sa{};
    sa.src = op; sa.K = K; sa.T = T; sa.tiles = out.tiles; sa.Kb = out.Kb;
    sa.out = out.planes.as<uint16_t>(); sa.emax = out.emax.as<int>(); sa.err = err;
    if (op.sk == 1) {
        const int64_t warps = std::min<int64_t>(op.rows, 64ll * sm_count());
        emax_contig_kernel<<<(unsigned)ceil_div(warps * 32, 256), 256, 0, stream>>>(op, K, out.emax.as<int>(), err);
        RT_TRY(check_launch("emax_contig_kernel"));
        dim3 grid((unsigned)out.tiles, (unsigned)ceil_div(K, SK));
        slice_contig_kernel<S><<<grid, 256, 0, stream>>>(sa);
        RT_TRY(check_launch("slice_contig_kernel"));
    } else if (op.s0 == 1) {
        RT_CUDA_TRY(cudaMemsetAsync(out.emax.p, 0, sizeof(int) * (size_t)op.rows, stream));
        const int64_t kspan = 512;
        dim3 g1((unsigned)ceil_div(op.rows, 256), (unsigned)ceil_div(K, kspan));
        emax_strided_kernel<<<g1, 256, 0, stream>>>(op, K, kspan, out.emax.as<int>(), err);
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

template <int S>
rt_status run(const OzGemm& g, cudaStream_t stream) {
    static bool attr_done = false;
    if (!attr_done) {
        set_smem_attr<S>();
        attr_done = true;
    }
    Operand A{g.A.p, g.A.rows, g.A.div, g.A.s0, g.A.s1, g.A.sk};
    Operand B{g.B.p, g.B.rows, g.B.div, g.B.s0, g.B.s1, g.B.sk};
    Sliced sa, sb;
    const bool reuse = g.b_is_a;
    // Slicing is HBM-bound: count bytes (8 read + 2*S written per element).
    const double slice_bytes = (double)(A.rows + (reuse ? 0 : B.rows)) * (double)g.K * (8.0 + 2.0 * S);
    prof_begin(PROF_OZ_SLICE, stream);
    RT_TRY(slice_operand<S>(A, g.K, TM, sa, stream));
    if (!reuse) RT_TRY(slice_operand<S>(B, g.K, TN, sb, stream));
    prof_end(PROF_OZ_SLICE, stream, slice_bytes);

    GemmArgs a{};
    a.a_slices = sa.planes.as<uint8_t>();
    a.a_s_stride = TM * KB * 2;
    a.a_kb_stride = (int64_t)S * TM * KB * 2;
    a.a_tile_stride = sa.Kb * a.a_kb_stride;
    if (reuse) {
        a.b_slices = sa.planes.as<uint8_t>();
        a.b_tile2_stride = a.a_tile_stride;
        a.b_half_stride = TN * KB * 2;
        a.b_kb_stride = a.a_kb_stride;
        a.b_s_stride = a.a_s_stride;
        a.eb = sa.emax.as<int>();
    } else {
        a.b_slices = sb.planes.as<uint8_t>();
        a.b_s_stride = TN * KB * 2;
        a.b_kb_stride = (int64_t)S * TN * KB * 2;
        a.b_half_stride = sb.Kb * a.b_kb_stride;
        a.b_tile2_stride = 2 * a.b_half_stride;
        a.eb = sb.emax.as<int>();
    }
    a.ea = sa.emax.as<int>();
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

    // Split the chunk range across CTAs when there are too few tiles to fill the
    // GPU; pick the split count whose CTA total best fills whole waves.
    const int64_t tiles = a.tiles_m * a.tiles_n;
    int64_t active = tiles;
    if (g.symmetric) {
        active = 0;
        for (int64_t tm = 0; tm < a.tiles_m; ++tm)
            for (int64_t tn = 0; tn < a.tiles_n; ++tn)
                if (tn * TN + TN - 1 >= tm * TM) ++active;
    }
    int64_t splits = 1;
    const int64_t sms = sm_count();
    if (active < sms && a.nchunks > 1) {
        double best = 0.0;
        for (int64_t w = 1; w <= 4; ++w) {
            const int64_t sp = std::min<int64_t>(a.nchunks, std::max<int64_t>(1, (w * sms) / active));
            const double eff = (double)(active * sp) / (double)(ceil_div(active * sp, sms) * sms);
            if (eff > best + 0.02) { best = eff; splits = sp; }
        }
    }
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

    ScratchBuf part;
    if (splits > 1) {
        RT_TRY(scratch_alloc(part, sizeof(int64_t) * (size_t)splits * a.tiles_m * TM * a.tiles_n * TN, stream));
        a.partial = part.as<int64_t>();
    }
    constexpr int smem = num_stages(S) * stage_bytes(S) + 256;
    dim3 grid((unsigned)std::min<int64_t>(tiles * splits, sms));
    // Algorithmic tensor work: S(S+1)/2 digit-pair products of 2*M*N*K each
    // (half of the square for the symmetric product).
    const double pair_flops = 2.0 * (double)a.M * (double)a.N * (double)g.K * (g.symmetric ? 0.5 : 1.0);
    prof_begin(PROF_OZ_GEMM, stream);
    oz_gemm_kernel<S><<<grid, NTHREADS, smem, stream>>>(a);
    prof_end(PROF_OZ_GEMM, stream, pair_flops * S * (S + 1) / 2);
    RT_TRY(check_launch("oz_gemm_kernel"));
    if (splits > 1) {
        oz_finalize_kernel<S><<<4 * sm_count(), 256, 0, stream>>>(a);
        RT_TRY(check_launch("oz_finalize_kernel"));
    }
    if (g.symmetric) {
        mirror_kernel<<<4 * sm_count(), 256, 0, stream>>>(a.out, a.M);
        RT_TRY(check_launch("mirror_kernel"));
    }
    return RT_OK;
}

}  // namespace oz

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
