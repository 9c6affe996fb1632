// fp64.cu - the plain float64 form of the RI path.
//
// GB300 executes float64 on the CUDA cores (DFMA); its tensor cores have no
// float64 kind and the legacy DMMA path is slower than DFMA on this part
// (1.05 vs 1.20 TFLOP/s measured).  The plain form is therefore one
// register-tiled DFMA GEMM service (batched, strided, optional split-K) on
// which every contraction is composed, plus two DFMA streaming kernels for
// RI-J and a fixed-order reduction for the exchange energy.
#include <algorithm>
#include <deque>
#include <mutex>

#include "rt_internal.cuh"
#include "../../include/rt_synth.h"

namespace rt {

namespace {

constexpr int BM = 64, BN = 64, BK = 16, NT = 256;

struct GemmArgs {
    int64_t m, n, k;
    double alpha, beta;
    const double* A;
    int64_t lda, sA;
    const double* B;
    int64_t ldb, sB;
    double* C;
    int64_t rsC, csC, bsC;
    int64_t batch;
    int64_t tiles_m, tiles_n;
    int splitk;
    int64_t kchunk;
    double* partial;  // splitk > 1: [splitk][batch][m*n]
    int64_t a_div, a_s1;  // composite A rows (kNoDiv: plain)
    int64_t c_md, c_ms1;  // composite C rows
};

// Offset of A's row gm (opa 'N': element (gm, k) at offset + k*lda; 'T': at offset + k).
template <bool TA>
__device__ __forceinline__ int64_t a_row_offset(const GemmArgs& g, int64_t gm) {
    if (g.a_div == kNoDiv) return TA ? gm * g.lda : gm;
    const int64_t lo = gm % g.a_div, hi = gm / g.a_div;
    return (TA ? lo * g.lda : lo) + hi * g.a_s1;
}
__device__ __forceinline__ int64_t c_row_offset(const GemmArgs& g, int64_t gm) {
    if (g.c_md == kNoDiv) return gm * g.rsC;
    return (gm % g.c_md) * g.rsC + (gm / g.c_md) * g.c_ms1;
}

// One BMT x BNT output tile per CTA (64x64; 128x32, 32x128, 256x16 or 16x256
// for a narrow side), 16-deep k slices staged through shared memory, 4x4 outputs per thread.
// Thread (tx, ty) owns rows tx + TXN*i and columns ty + TYN*j, so a warp reads
// at most 32 distinct A values and a few distinct B values per k step
// (broadcasts, no bank conflicts beyond the 2-wavefront double access).
template <bool TA, bool TB, int BMT, int BNT>
__device__ __forceinline__ void dgemm_tile_body(const GemmArgs& g, int64_t tile, int64_t b_first, int64_t b_step,
                                                int split) {
    constexpr int TXN = BMT / 4, TYN = BNT / 4;
    static_assert(TXN * TYN == NT, "4x4 outputs per thread");
    __shared__ double As[BK][BMT + 1];
    __shared__ double Bs[BK][BNT + 1];
    const int tid = threadIdx.x;
    const int tx = tid % TXN, ty = tid / TXN;
    const int64_t tm = tile % g.tiles_m, tn = tile / g.tiles_m;
    const int64_t m0 = tm * BMT, n0 = tn * BNT;
    const int64_t k0 = (int64_t)split * g.kchunk;
    const int64_t k1 = min(g.k, k0 + g.kchunk);

    // Row offsets of the A elements this thread stages (fixed for the tile).
    constexpr int RA = (BMT * BK) / NT;
    int64_t aoff[TA ? RA : 1];
#pragma unroll
    for (int r = 0; r < (TA ? RA : 1); ++r) {
        const int mi = TA ? (tid >> 4) + 16 * r : tid % BMT;
        aoff[r] = a_row_offset<TA>(g, min(m0 + mi, g.m - 1));
    }
    for (int64_t b = b_first; b < g.batch; b += b_step) {
        const double* A = g.A + b * g.sA;
        const double* B = g.B + b * g.sB;
        double acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

        for (int64_t kk = k0; kk < k1; kk += BK) {
            // Stage A tile (BMT x BK) as As[k][m]; consecutive threads read consecutive addresses.
#pragma unroll
            for (int r = 0; r < (BMT * BK) / NT; ++r) {
                int mi, ki;
                if (!TA) { mi = tid % BMT; ki = tid / BMT + (NT / BMT) * r; }
                else { ki = tid & 15; mi = (tid >> 4) + 16 * r; }
                const int64_t gm = m0 + mi, gk = kk + ki;
                double v = 0.0;
                if (gm < g.m && gk < k1) v = TA ? A[aoff[TA ? r : 0] + gk] : A[aoff[0] + gk * g.lda];
                As[ki][mi] = v;
            }
            // Stage B tile (BK x BNT) as Bs[k][n].
#pragma unroll
            for (int r = 0; r < (BNT * BK) / NT; ++r) {
                int ni, ki;
                if (!TB) { ki = tid & 15; ni = (tid >> 4) + 16 * r; }
                else { ni = tid % BNT; ki = tid / BNT + (NT / BNT) * r; }
                const int64_t gn = n0 + ni, gk = kk + ki;
                double v = 0.0;
                if (gn < g.n && gk < k1) v = TB ? B[gn + gk * g.ldb] : B[gk + gn * g.ldb];
                Bs[ki][ni] = v;
            }
            __syncthreads();
#pragma unroll
            for (int q = 0; q < BK; ++q) {
                double a[4], bb[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) a[i] = As[q][tx + TXN * i];
#pragma unroll
                for (int j = 0; j < 4; ++j) bb[j] = Bs[q][ty + TYN * j];
#pragma unroll
                for (int i = 0; i < 4; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], bb[j], acc[i][j]);
            }
            __syncthreads();
        }

#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int64_t gm = m0 + tx + TXN * i;
            if (gm >= g.m) continue;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int64_t gn = n0 + ty + TYN * j;
                if (gn >= g.n) continue;
                if (g.splitk > 1) {
                    g.partial[((int64_t)split * g.batch + b) * g.m * g.n + gm + gn * g.m] = acc[i][j];
                } else {
                    double* c = g.C + c_row_offset(g, gm) + gn * g.csC + b * g.bsC;
                    double v = g.alpha * acc[i][j];
                    if (g.beta != 0.0) v = fma(g.beta, *c, v);
                    *c = v;
                }
            }
        }
    }
}

// Tile shapes: 0 = 64x64, 1 = 128x32 (n <= 32), 2 = 32x128 (m <= 32),
// 3 = 256x16 (n <= 16), 4 = 16x256 (m <= 16).
constexpr int kShapes = 5;
constexpr int tile_bm(int shape) {
    return shape == 1 ? 128 : shape == 2 ? 32 : shape == 3 ? 256 : shape == 4 ? 16 : 64;
}
constexpr int tile_bn(int shape) {
    return shape == 1 ? 32 : shape == 2 ? 128 : shape == 3 ? 16 : shape == 4 ? 256 : 64;
}
inline int pick_shape(int64_t m, int64_t n) {
    if (n <= 16 && m > 64) return 3;
    if (m <= 16 && n > 64) return 4;
    if (n <= 32 && m > 32) return 1;
    if (m <= 32 && n > 32) return 2;
    return 0;
}

template <bool TA, bool TB, int SH>
__global__ void __launch_bounds__(NT) dgemm_tile_kernel(GemmArgs g) {
    dgemm_tile_body<TA, TB, tile_bm(SH), tile_bn(SH)>(g, blockIdx.x, blockIdx.y, gridDim.y, blockIdx.z);
}

// Several float64 GEMMs (same op pair and tile shape) in one launch: block x
// enumerates (problem, tile, batch item) through the prefix sums of tiles * batch.
constexpr int kMaxGroupF64 = 64;
struct GroupF64 {
    int n;
    int64_t prefix[kMaxGroupF64 + 1];
    GemmArgs a[kMaxGroupF64];
};

static_assert(sizeof(GroupF64) <= 32000, "kernel parameter block too large");

template <bool TA, bool TB, int SH>
__global__ void __launch_bounds__(NT) dgemm_group_kernel(const __grid_constant__ GroupF64 G) {
    const int64_t blk = blockIdx.x;
    int p = 0;
    while (blk >= G.prefix[p + 1]) ++p;
    const GemmArgs& g = G.a[p];
    const int64_t local = blk - G.prefix[p];
    const int64_t tiles = g.tiles_m * g.tiles_n;
    const int64_t per_split = tiles * g.batch;
    const int64_t rem = local % per_split;
    dgemm_tile_body<TA, TB, tile_bm(SH), tile_bn(SH)>(g, rem % tiles, rem / tiles, g.batch,
                                                      (int)(local / per_split));
}

// Deterministic split-K reduction of several grouped products (those with
// splitk > 1): block x enumerates their output elements through prefix sums.
__global__ void dgemm_splitk_reduce_group(const __grid_constant__ GroupF64 G) {
    const int64_t total = G.prefix[G.n];
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        int p = 0;
        while (idx >= G.prefix[p + 1]) ++p;
        const GemmArgs& g = G.a[p];
        const int64_t e0 = idx - G.prefix[p];
        const int64_t mn = g.m * g.n;
        const int64_t b = e0 / mn, e = e0 % mn;
        const int64_t i = e % g.m, j = e / g.m;
        double s = 0.0;
        for (int z = 0; z < g.splitk; ++z) s += g.partial[((int64_t)z * g.batch + b) * mn + e];
        double* c = g.C + c_row_offset(g, i) + j * g.csC + b * g.bsC;
        double v = g.alpha * s;
        if (g.beta != 0.0) v = fma(g.beta, *c, v);
        *c = v;
    }
}

template <int SH>
void launch_tile(bool ta, bool tb, dim3 grid, const GemmArgs& g, cudaStream_t stream) {
    if (!ta && !tb) dgemm_tile_kernel<false, false, SH><<<grid, NT, 0, stream>>>(g);
    else if (ta && !tb) dgemm_tile_kernel<true, false, SH><<<grid, NT, 0, stream>>>(g);
    else if (!ta && tb) dgemm_tile_kernel<false, true, SH><<<grid, NT, 0, stream>>>(g);
    else dgemm_tile_kernel<true, true, SH><<<grid, NT, 0, stream>>>(g);
}

template <int SH>
void launch_group(bool ta, bool tb, unsigned blocks, const GroupF64& G, cudaStream_t stream) {
    if (!ta && !tb) dgemm_group_kernel<false, false, SH><<<blocks, NT, 0, stream>>>(G);
    else if (ta && !tb) dgemm_group_kernel<true, false, SH><<<blocks, NT, 0, stream>>>(G);
    else if (!ta && tb) dgemm_group_kernel<false, true, SH><<<blocks, NT, 0, stream>>>(G);
    else dgemm_group_kernel<true, true, SH><<<blocks, NT, 0, stream>>>(G);
}

// Deterministic split-K reduction: fixed summation order over the splits.
__global__ void dgemm_splitk_reduce(GemmArgs g) {
    const int64_t mn = g.m * g.n;
    const int64_t total = mn * g.batch;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = idx / mn, e = idx % mn;
        const int64_t i = e % g.m, j = e / g.m;
        double s = 0.0;
        for (int z = 0; z < g.splitk; ++z) s += g.partial[((int64_t)z * g.batch + b) * mn + e];
        double* c = g.C + c_row_offset(g, i) + j * g.csC + b * g.bsC;
        double v = g.alpha * s;
        if (g.beta != 0.0) v = fma(g.beta, *c, v);
        *c = v;
    }
}

__global__ void scale_kernel(GemmArgs g) {
    // k == 0: C = beta * C
    const int64_t mn = g.m * g.n, total = mn * g.batch;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = idx / mn, e = idx % mn;
        double* c = g.C + c_row_offset(g, e % g.m) + (e / g.m) * g.csC + b * g.bsC;
        *c = g.beta == 0.0 ? 0.0 : g.beta * *c;
    }
}

}  // namespace

rt_status gemm_f64(const GemmF64& q, cudaStream_t stream) {
    RT_REQUIRE(q.m >= 0 && q.n >= 0 && q.k >= 0 && q.batch >= 0, "gemm_f64: negative size");
    RT_REQUIRE((q.opa == 'N' || q.opa == 'T') && (q.opb == 'N' || q.opb == 'T'), "gemm_f64: op must be N or T");
    if (q.m == 0 || q.n == 0 || q.batch == 0) return RT_OK;
    GemmArgs g{};
    g.m = q.m; g.n = q.n; g.k = q.k; g.alpha = q.alpha; g.beta = q.beta;
    g.A = q.A; g.lda = q.lda; g.sA = q.sA; g.B = q.B; g.ldb = q.ldb; g.sB = q.sB;
    g.C = q.C; g.rsC = q.rsC; g.csC = q.csC; g.bsC = q.bsC; g.batch = q.batch;
    g.a_div = q.a_div; g.a_s1 = q.a_s1; g.c_md = q.c_md; g.c_ms1 = q.c_ms1;
    const int shape = pick_shape(q.m, q.n);
    g.tiles_m = ceil_div(q.m, (int64_t)tile_bm(shape));
    g.tiles_n = ceil_div(q.n, (int64_t)tile_bn(shape));
    if (q.k == 0) {
        scale_kernel<<<1024, 256, 0, stream>>>(g);
        return check_launch("gemm_f64 scale");
    }
    int splitk = q.splitk < 1 ? 1 : q.splitk;
    int64_t kchunk = ceil_div(ceil_div(q.k, splitk), BK) * BK;
    splitk = (int)ceil_div(q.k, kchunk);
    g.splitk = splitk;
    g.kchunk = kchunk;
    ScratchBuf part;
    if (splitk > 1) {
        RT_TRY(scratch_alloc(part, sizeof(double) * (size_t)splitk * q.batch * q.m * q.n, stream));
        g.partial = part.as<double>();
    }
    dim3 grid((unsigned)(g.tiles_m * g.tiles_n), (unsigned)(q.batch < 65535 ? q.batch : 65535), (unsigned)splitk);
    const bool ta = q.opa == 'T', tb = q.opb == 'T';
    prof_begin(PROF_DGEMM, stream);
    switch (shape) {
        case 1: launch_tile<1>(ta, tb, grid, g, stream); break;
        case 2: launch_tile<2>(ta, tb, grid, g, stream); break;
        case 3: launch_tile<3>(ta, tb, grid, g, stream); break;
        case 4: launch_tile<4>(ta, tb, grid, g, stream); break;
        default: launch_tile<0>(ta, tb, grid, g, stream); break;
    }
    prof_end(PROF_DGEMM, stream, 2.0 * (double)q.m * (double)q.n * (double)q.k * (double)q.batch);
    RT_TRY(check_launch("dgemm_tile_kernel"));
    if (splitk > 1) {
        dgemm_splitk_reduce<<<2 * sm_count(), 256, 0, stream>>>(g);
        RT_TRY(check_launch("dgemm_splitk_reduce"));
    }
    return RT_OK;
}

rt_status gemm_f64_many(const GemmF64* qs, int n, cudaStream_t stream) {
    // Group by op pair and tile shape; each group goes out in launches of up to
    // kMaxGroupF64 products.
    for (int i = 0; i < n; ++i)
        RT_REQUIRE(qs[i].m >= 0 && qs[i].n >= 0 && qs[i].k > 0 && qs[i].batch >= 0, "gemm_f64_many: bad size");
    std::deque<ScratchBuf> parts;  // split-K partials, released after the reductions (stream order)
    for (int op = 0; op < 4; ++op) {
        const bool ta = op & 1, tb = op & 2;
        for (int shape = 0; shape < kShapes; ++shape) {
            GroupF64 G;
            G.n = 0;
            G.prefix[0] = 0;
            double flops = 0.0;
            auto flush = [&]() -> rt_status {
                if (G.n == 0) return RT_OK;
                for (int i = G.n; i < kMaxGroupF64; ++i) G.prefix[i + 1] = G.prefix[G.n];
                const int64_t blocks = G.prefix[G.n];
                if (blocks > 0) {
                    RT_REQUIRE(blocks < (int64_t)INT32_MAX, "gemm_f64_many: too many tiles for one launch");
                    prof_begin(PROF_DGEMM, stream);
                    switch (shape) {
                        case 1: launch_group<1>(ta, tb, (unsigned)blocks, G, stream); break;
                        case 2: launch_group<2>(ta, tb, (unsigned)blocks, G, stream); break;
                        case 3: launch_group<3>(ta, tb, (unsigned)blocks, G, stream); break;
                        case 4: launch_group<4>(ta, tb, (unsigned)blocks, G, stream); break;
                        default: launch_group<0>(ta, tb, (unsigned)blocks, G, stream); break;
                    }
                    prof_end(PROF_DGEMM, stream, flops);
                    RT_TRY(check_launch("dgemm_group_kernel"));
                    // One deterministic reduction for every split product of the launch.
                    GroupF64 R;
                    R.n = 0;
                    R.prefix[0] = 0;
                    for (int i = 0; i < G.n; ++i) {
                        if (G.a[i].splitk <= 1) continue;
                        R.a[R.n] = G.a[i];
                        R.prefix[R.n + 1] = R.prefix[R.n] + G.a[i].m * G.a[i].n * G.a[i].batch;
                        ++R.n;
                    }
                    if (R.n > 0) {
                        for (int i = R.n; i < kMaxGroupF64; ++i) R.prefix[i + 1] = R.prefix[R.n];
                        dgemm_splitk_reduce_group<<<2 * sm_count(), 256, 0, stream>>>(R);
                        RT_TRY(check_launch("dgemm_splitk_reduce_group"));
                    }
                }
                G.n = 0;
                flops = 0.0;
                return RT_OK;
            };
            for (int i = 0; i < n; ++i) {
                const GemmF64& q = qs[i];
                if ((q.opa == 'T') != ta || (q.opb == 'T') != tb) continue;
                if (q.m == 0 || q.n == 0 || q.batch == 0) continue;
                if (pick_shape(q.m, q.n) != shape) continue;
                GemmArgs& g = G.a[G.n];
                g = GemmArgs{};
                g.m = q.m; g.n = q.n; g.k = q.k; g.alpha = q.alpha; g.beta = q.beta;
                g.A = q.A; g.lda = q.lda; g.sA = q.sA; g.B = q.B; g.ldb = q.ldb; g.sB = q.sB;
                g.C = q.C; g.rsC = q.rsC; g.csC = q.csC; g.bsC = q.bsC; g.batch = q.batch;
                g.a_div = q.a_div; g.a_s1 = q.a_s1; g.c_md = q.c_md; g.c_ms1 = q.c_ms1;
    g.a_div = q.a_div; g.a_s1 = q.a_s1; g.c_md = q.c_md; g.c_ms1 = q.c_ms1;
                g.tiles_m = ceil_div(q.m, (int64_t)tile_bm(shape));
                g.tiles_n = ceil_div(q.n, (int64_t)tile_bn(shape));
                const int want = q.splitk < 1 ? 1 : q.splitk;
                g.kchunk = std::max<int64_t>(BK, ceil_div(ceil_div(q.k, want), BK) * BK);
                g.splitk = (int)std::max<int64_t>(1, ceil_div(q.k, g.kchunk));
                if (g.splitk > 1) {
                    parts.emplace_back();
                    RT_TRY(scratch_alloc(parts.back(),
                                         sizeof(double) * (size_t)g.splitk * q.batch * q.m * q.n, stream));
                    g.partial = parts.back().as<double>();
                }
                G.prefix[G.n + 1] = G.prefix[G.n] + g.tiles_m * g.tiles_n * q.batch * g.splitk;
                flops += 2.0 * (double)q.m * (double)q.n * (double)q.k * (double)q.batch;
                ++G.n;
                if (G.n == kMaxGroupF64) RT_TRY(flush());
            }
            RT_TRY(flush());
        }
    }
    return RT_OK;
}

// ------------------------------------------------------------------ RI-J --

namespace {

// w[P] = sum_e B[e + n2*P] * D[e]; one CTA per slab, fixed-order block tree.
__global__ void __launch_bounds__(256) rij_w_kernel(const double* __restrict__ B, const double* __restrict__ D,
                                                    int64_t n2, int naux, double* __restrict__ w) {
    __shared__ double red[8];
    // 16-byte loads when every slab starts 16-byte aligned; four independent
    // accumulators keep eight loads in flight per thread.
    const bool vec = (n2 & 1) == 0 && ((uintptr_t)B & 15) == 0 && ((uintptr_t)D & 15) == 0;
    for (int P = blockIdx.x; P < naux; P += gridDim.x) {
        const double* b = B + (int64_t)P * n2;
        double s[4] = {0.0, 0.0, 0.0, 0.0};
        if (vec) {
            const double2* b2 = reinterpret_cast<const double2*>(b);
            const double2* d2 = reinterpret_cast<const double2*>(D);
            const int64_t h = n2 / 2;
            int64_t e = threadIdx.x;
            for (; e + 768 < h; e += 1024) {
                double2 x[4], y[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    x[u] = b2[e + 256 * u];
                    y[u] = d2[e + 256 * u];
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) s[u] = fma(x[u].y, y[u].y, fma(x[u].x, y[u].x, s[u]));
            }
            for (; e < h; e += 256) {
                const double2 x = b2[e], y = d2[e];
                s[0] = fma(x.y, y.y, fma(x.x, y.x, s[0]));
            }
        } else {
            for (int64_t e = threadIdx.x; e < n2; e += 256) s[0] = fma(b[e], D[e], s[0]);
        }
        double t0 = (s[0] + s[1]) + (s[2] + s[3]);
        for (int o = 16; o > 0; o >>= 1) t0 += __shfl_xor_sync(0xffffffffu, t0, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t0;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = threadIdx.x < 8 ? red[threadIdx.x] : 0.0;
            for (int o = 4; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (threadIdx.x == 0) w[P] = t;
        }
        __syncthreads();
    }
}

// J[e] = sum_P w[P] * B[e + n2*P]; each thread owns two adjacent elements and
// walks the slabs (coalesced 16-byte loads across the warp).
__global__ void __launch_bounds__(256) rij_j_kernel(const double* __restrict__ B, const double* __restrict__ w,
                                                    int64_t n2, int naux, double* __restrict__ J) {
    __shared__ double ws[1024];
    const int64_t e = 2 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
    double a0 = 0.0, a1 = 0.0, c0 = 0.0, c1 = 0.0;
    for (int P0 = 0; P0 < naux; P0 += 1024) {
        const int np = min(1024, naux - P0);
        __syncthreads();
        for (int t = threadIdx.x; t < np; t += blockDim.x) ws[t] = w[P0 + t];
        __syncthreads();
        if (e + 1 < n2) {
            const double2* b2 = reinterpret_cast<const double2*>(B + e + (int64_t)P0 * n2);
            const int64_t st = n2 / 2;
            int p = 0;
            // eight slabs in flight per thread
            for (; p + 7 < np; p += 8) {
                double2 x[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) x[u] = b2[(int64_t)(p + u) * st];
#pragma unroll
                for (int u = 0; u < 8; u += 2) {
                    a0 = fma(ws[p + u], x[u].x, a0);
                    a1 = fma(ws[p + u], x[u].y, a1);
                    c0 = fma(ws[p + u + 1], x[u + 1].x, c0);
                    c1 = fma(ws[p + u + 1], x[u + 1].y, c1);
                }
            }
            for (; p + 1 < np; p += 2) {
                double2 x = b2[(int64_t)p * st], y = b2[(int64_t)(p + 1) * st];
                a0 = fma(ws[p], x.x, a0);
                a1 = fma(ws[p], x.y, a1);
                c0 = fma(ws[p + 1], y.x, c0);
                c1 = fma(ws[p + 1], y.y, c1);
            }
            if (p < np) {
                double2 x = b2[(int64_t)p * st];
                a0 = fma(ws[p], x.x, a0);
                a1 = fma(ws[p], x.y, a1);
            }
        } else if (e < n2) {
            for (int p = 0; p < np; ++p) a0 = fma(ws[p], B[e + (int64_t)(P0 + p) * n2], a0);
        }
    }
    if (e + 1 < n2) {
        J[e] = a0 + c0;
        J[e + 1] = a1 + c1;
    } else if (e < n2) {
        J[e] = a0;
    }
}

// Same, for odd n2 where 16-byte alignment of every slab cannot be assumed.
__global__ void __launch_bounds__(256) rij_j_kernel_scalar(const double* __restrict__ B,
                                                           const double* __restrict__ w, int64_t n2, int naux,
                                                           double* __restrict__ J) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n2) return;
    double a0 = 0.0, a1 = 0.0;
    int p = 0;
    for (; p + 1 < naux; p += 2) {
        a0 = fma(w[p], B[e + (int64_t)p * n2], a0);
        a1 = fma(w[p + 1], B[e + (int64_t)(p + 1) * n2], a1);
    }
    if (p < naux) a0 = fma(w[p], B[e + (int64_t)p * n2], a0);
    J[e] = a0 + a1;
}

// -tr(D K) with one CTA and a fixed reduction tree (bitwise reproducible).
__global__ void __launch_bounds__(1024) exchange_kernel(const double* __restrict__ D, const double* __restrict__ K,
                                                        int64_t n2, double* __restrict__ out) {
    __shared__ double red[32];
    double s = 0.0, c = 0.0;  // Kahan-compensated per-thread partial
    for (int64_t e = threadIdx.x; e < n2; e += blockDim.x) {
        double y = fma(D[e], K[e], -c);
        double t = s + y;
        c = (t - s) - y;
        s = t;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = red[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) *out = -t;
    }
}

__global__ void synth_coef_kernel(uint64_t seed, int nb, double* M) {
    const int64_t total = (int64_t)nb * nb;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x)
        M[idx] = rt_coef_seed_elem(seed, idx % nb, idx / nb);
}

// ---- RI-J on symmetric slabs (B^P and D symmetric): only entries mu <= nu
// are read, and each product is formed once.  Both passes are bound by the
// float64 FMA rate, so halving the products halves the time.

// D2[mu, nu] = 2 D[mu, nu] above the diagonal, D[mu, mu] on it, 0 below:
// w_P = sum_{mu <= nu} D2[mu, nu] B^P[mu, nu].
__global__ void rij_d2_kernel(const double* __restrict__ D, int nb, double* __restrict__ D2) {
    const int64_t n2 = (int64_t)nb * nb;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n2; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t mu = e % nb, nu = e / nb;
        D2[e] = mu < nu ? 2.0 * D[e] : (mu == nu ? D[e] : 0.0);
    }
}

// w[P] for slab P, one block per slab: warp c takes the column pairs
// (c, nb-1-c), (c+8, nb-9-c), ... (nb+1 upper entries per pair), lanes run down
// each column's upper part with four loads in flight; fixed-order reduction.
__global__ void __launch_bounds__(256) rij_w_sym_kernel(const double* __restrict__ B, const double* __restrict__ D2,
                                                        int nb, int naux, double* __restrict__ w) {
    __shared__ double red[8];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t n2 = (int64_t)nb * nb;
    const int half = (nb + 1) / 2;
    for (int P = blockIdx.x; P < naux; P += gridDim.x) {
        const double* b = B + (int64_t)P * n2;
        double s[4] = {0.0, 0.0, 0.0, 0.0};
        for (int c = warp; c < half; c += 8) {
#pragma unroll 1
            for (int side = 0; side < 2; ++side) {
                const int nu = side ? nb - 1 - c : c;
                if (side && nu == c) break;
                const double* bc = b + (int64_t)nb * nu;
                const double* dc = D2 + (int64_t)nb * nu;
                int mu = lane;
                for (; mu + 96 <= nu; mu += 128) {
                    double x[4], y[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        x[u] = bc[mu + 32 * u];
                        y[u] = dc[mu + 32 * u];
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) s[u] = fma(x[u], y[u], s[u]);
                }
                for (; mu <= nu; mu += 32) s[0] = fma(bc[mu], dc[mu], s[0]);
            }
        }
        double t0 = (s[0] + s[1]) + (s[2] + s[3]);
        for (int o = 16; o > 0; o >>= 1) t0 += __shfl_xor_sync(0xffffffffu, t0, o);
        if (lane == 0) red[warp] = t0;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = threadIdx.x < 8 ? red[threadIdx.x] : 0.0;
            for (int o = 4; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
            if (threadIdx.x == 0) w[P] = t;
        }
        __syncthreads();
    }
}

// Column nu and row mu of packed upper-triangle index t = nu (nu + 1) / 2 + mu.
__device__ __forceinline__ void tri_index(int64_t t, int& mu, int& nu) {
    int64_t v = (int64_t)((sqrt(8.0 * (double)t + 1.0) - 1.0) * 0.5);
    while (v * (v + 1) / 2 > t) --v;
    while ((v + 1) * (v + 2) / 2 <= t) ++v;
    nu = (int)v;
    mu = (int)(t - v * (v + 1) / 2);
}

// Partial J over the slab range of split blockIdx.y: each thread owns packed
// upper-triangle entries t and t+1, part[split][t] = sum_P w[P] B^P[mu, nu].
__global__ void __launch_bounds__(256) rij_j_sym_kernel(const double* __restrict__ B, const double* __restrict__ w,
                                                        int nb, int naux, int64_t T, int pspan,
                                                        double* __restrict__ part) {
    __shared__ double ws[1024];
    const int64_t n2 = (int64_t)nb * nb;
    const int64_t t0 = 2 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x);
    const bool v0 = t0 < T, v1 = t0 + 1 < T;
    int mu, nu;
    int64_t o0 = 0, o1 = 0;
    if (v0) {
        tri_index(t0, mu, nu);
        o0 = mu + (int64_t)nb * nu;
    }
    if (v1) {
        tri_index(t0 + 1, mu, nu);
        o1 = mu + (int64_t)nb * nu;
    }
    const int Pb = blockIdx.y * pspan, Pe = min(naux, Pb + pspan);
    double a0 = 0.0, a1 = 0.0, c0 = 0.0, c1 = 0.0;
    for (int P0 = Pb; P0 < Pe; P0 += 1024) {
        const int np = min(1024, Pe - P0);
        __syncthreads();
        for (int t = threadIdx.x; t < np; t += blockDim.x) ws[t] = w[P0 + t];
        __syncthreads();
        if (!v0) continue;
        const double* b0 = B + o0 + (int64_t)P0 * n2;
        const double* b1 = B + (v1 ? o1 : o0) + (int64_t)P0 * n2;
        int p = 0;
        for (; p + 3 < np; p += 4) {
            double x[4], y[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                x[u] = b0[(int64_t)(p + u) * n2];
                y[u] = b1[(int64_t)(p + u) * n2];
            }
#pragma unroll
            for (int u = 0; u < 4; u += 2) {
                a0 = fma(ws[p + u], x[u], a0);
                a1 = fma(ws[p + u], y[u], a1);
                c0 = fma(ws[p + u + 1], x[u + 1], c0);
                c1 = fma(ws[p + u + 1], y[u + 1], c1);
            }
        }
        for (; p < np; ++p) {
            a0 = fma(ws[p], b0[(int64_t)p * n2], a0);
            a1 = fma(ws[p], b1[(int64_t)p * n2], a1);
        }
    }
    if (v0) part[(int64_t)blockIdx.y * T + t0] = a0 + c0;
    if (v1) part[(int64_t)blockIdx.y * T + t0 + 1] = a1 + c1;
}

// J[mu, nu] = J[nu, mu] = the splits' partials summed in order.
__global__ void rij_j_sym_finish(const double* __restrict__ part, int nb, int64_t T, int splits,
                                 double* __restrict__ J) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < T; t += (int64_t)gridDim.x * blockDim.x) {
        double a = 0.0;
        for (int z = 0; z < splits; ++z) a += part[(int64_t)z * T + t];
        int mu, nu;
        tri_index(t, mu, nu);
        J[mu + (int64_t)nb * nu] = a;
        J[nu + (int64_t)nb * mu] = a;
    }
}

__global__ void synth_kernel(uint64_t seed, int nb, int P0, int64_t total, double* B) {
    const int64_t nb2 = (int64_t)nb * nb;
    for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (int64_t)gridDim.x * blockDim.x) {
        const int64_t P = idx / nb2, r = idx % nb2;
        const int64_t mu = r % nb, nu = r / nb;
        B[idx] = rt_ri3ao_elem(seed, P0 + P, mu, nu);
    }
}

}  // namespace

rt_status ri_j_fp64(const double* B, const double* D, int nb, int naux, double* w, double* J,
                    cudaStream_t stream) {
    const int64_t n2 = (int64_t)nb * nb;
    ScratchBuf wbuf;
    if (!w) {
        RT_TRY(scratch_alloc(wbuf, sizeof(double) * (size_t)naux, stream));
        w = wbuf.as<double>();
    }
    rij_w_kernel<<<(unsigned)naux, 256, 0, stream>>>(B, D, n2, naux, w);
    RT_TRY(check_launch("rij_w_kernel"));
    if (J) {
        if ((n2 & 1) == 0 && ((uintptr_t)B & 15) == 0) {
            const int64_t threads = n2 / 2;
            rij_j_kernel<<<(unsigned)ceil_div(threads, 256), 256, 0, stream>>>(B, w, n2, naux, J);
        } else {
            rij_j_kernel_scalar<<<(unsigned)ceil_div(n2, 256), 256, 0, stream>>>(B, w, n2, naux, J);
        }
        RT_TRY(check_launch("rij_j_kernel"));
    }
    return RT_OK;
}

rt_status ri_j_fp64_symmetric(const double* B, const double* D, int nb, int naux, double* w, double* J,
                              cudaStream_t stream) {
    const int64_t n2 = (int64_t)nb * nb, T = (int64_t)nb * (nb + 1) / 2;
    ScratchBuf wbuf, d2buf, partbuf;
    if (!w) {
        RT_TRY(scratch_alloc(wbuf, sizeof(double) * (size_t)naux, stream));
        w = wbuf.as<double>();
    }
    RT_TRY(scratch_alloc(d2buf, sizeof(double) * (size_t)n2, stream));
    double* D2 = d2buf.as<double>();
    rij_d2_kernel<<<(unsigned)std::min<int64_t>(ceil_div(n2, 256), 4 * sm_count()), 256, 0, stream>>>(D, nb, D2);
    RT_TRY(check_launch("rij_d2_kernel"));
    rij_w_sym_kernel<<<(unsigned)naux, 256, 0, stream>>>(B, D2, nb, naux, w);
    RT_TRY(check_launch("rij_w_sym_kernel"));
    if (J) {
        // Split the slabs so that about eight blocks per SM run the J pass.
        const int64_t bx = ceil_div(ceil_div(T, (int64_t)2), (int64_t)256);
        const int splits = (int)std::max<int64_t>(1, std::min<int64_t>({ceil_div(8 * (int64_t)sm_count(), bx), 16, naux}));
        const int pspan = (int)ceil_div((int64_t)naux, (int64_t)splits);
        RT_TRY(scratch_alloc(partbuf, sizeof(double) * (size_t)(splits * T), stream));
        double* part = partbuf.as<double>();
        rij_j_sym_kernel<<<dim3((unsigned)bx, (unsigned)splits), 256, 0, stream>>>(B, w, nb, naux, T, pspan, part);
        RT_TRY(check_launch("rij_j_sym_kernel"));
        rij_j_sym_finish<<<(unsigned)std::min<int64_t>(ceil_div(T, 256), 4 * sm_count()), 256, 0, stream>>>(
            part, nb, T, splits, J);
        RT_TRY(check_launch("rij_j_sym_finish"));
    }
    return RT_OK;
}

rt_status exchange_energy(const double* D, const double* K, int nb, double* out, cudaStream_t stream) {
    exchange_kernel<<<1, 1024, 0, stream>>>(D, K, (int64_t)nb * nb, out);
    return check_launch("exchange_kernel");
}

rt_status synth_ri3ao(uint64_t seed, int nb, int P0, int nslab, double* B, cudaStream_t stream) {
    const int64_t total = (int64_t)nb * nb * nslab;
    if (total == 0) return RT_OK;
    synth_kernel<<<8 * sm_count(), 256, 0, stream>>>(seed, nb, P0, total, B);
    return check_launch("synth_kernel");
}

__global__ void synth_delta_kernel(uint64_t seed, int64_t nov, double* d) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nov; i += (int64_t)gridDim.x * blockDim.x)
        d[i] = rt_delta_elem(seed, i);
}

rt_status synth_delta(uint64_t seed, int64_t nov, double* d, cudaStream_t stream) {
    if (nov == 0) return RT_OK;
    synth_delta_kernel<<<2 * sm_count(), 256, 0, stream>>>(seed, nov, d);
    return check_launch("synth_delta_kernel");
}

rt_status synth_coef_seed(uint64_t seed, int nb, double* M, cudaStream_t stream) {
    if (nb <= 0) return RT_OK;
    synth_coef_kernel<<<sm_count(), 256, 0, stream>>>(seed, nb, M);
    return check_launch("synth_coef_kernel");
}

// Plain-form AO->MO transform: T^P = B^P C, then R^P = C^T T^P stored P-fastest.
// Slabs go through in blocks that keep the half-transformed scratch <= ~2 GB.
rt_status ri_ao2mo_fp64(const double* C, const double* B, double* R, int nb, int ns, int naux,
                        cudaStream_t stream) {
    const int64_t per = (int64_t)nb * ns;
    int64_t blk = (int64_t)((2ull << 30) / (sizeof(double) * (size_t)per));
    if (blk < 1) blk = 1;
    if (blk > naux) blk = naux;
    ScratchBuf tb;
    RT_TRY(scratch_alloc(tb, sizeof(double) * (size_t)(per * blk), stream));
    double* T = tb.as<double>();
    for (int64_t P0 = 0; P0 < naux; P0 += blk) {
        const int64_t np = std::min<int64_t>(blk, naux - P0);
        GemmF64 g1;
        g1.opa = 'N'; g1.opb = 'N'; g1.m = nb; g1.n = ns; g1.k = nb;
        g1.A = B + P0 * (int64_t)nb * nb; g1.lda = nb; g1.sA = (int64_t)nb * nb;
        g1.B = C; g1.ldb = nb; g1.sB = 0;
        g1.C = T; g1.rsC = 1; g1.csC = nb; g1.bsC = per; g1.batch = np;
        RT_TRY(gemm_f64(g1, stream));
        GemmF64 g2;
        g2.opa = 'T'; g2.opb = 'N'; g2.m = ns; g2.n = ns; g2.k = nb;
        g2.A = C; g2.lda = nb; g2.sA = 0;
        g2.B = T; g2.ldb = nb; g2.sB = per;
        g2.C = R + P0; g2.rsC = naux; g2.csC = (int64_t)naux * ns; g2.bsC = 1; g2.batch = np;
        RT_TRY(gemm_f64(g2, stream));
    }
    return RT_OK;
}

// Plain-form ov transform + RI-K with the shared half-transform X^P = B^P C_occ.
rt_status ri_ov_k_fp64(const double* C, const double* B, int nb, int naux, int nocc, int nvir, double* ov,
                       double* K, cudaStream_t stream) {
    const int64_t per = (int64_t)nb * nocc;
    ScratchBuf xb;
    RT_TRY(scratch_alloc(xb, sizeof(double) * (size_t)(per * naux), stream));
    double* X = xb.as<double>();
    GemmF64 g1;
    g1.opa = 'N'; g1.opb = 'N'; g1.m = nb; g1.n = nocc; g1.k = nb;
    g1.A = B; g1.lda = nb; g1.sA = (int64_t)nb * nb;
    g1.B = C; g1.ldb = nb; g1.sB = 0;
    g1.C = X; g1.rsC = 1; g1.csC = nb; g1.bsC = per; g1.batch = naux;
    RT_TRY(gemm_f64(g1, stream));
    if (ov && nvir > 0) {
        GemmF64 g2;
        g2.opa = 'T'; g2.opb = 'N'; g2.m = nocc; g2.n = nvir; g2.k = nb;
        g2.A = X; g2.lda = nb; g2.sA = per;
        g2.B = C + (int64_t)nb * nocc; g2.ldb = nb; g2.sB = 0;
        g2.C = ov; g2.rsC = 1; g2.csC = nocc; g2.bsC = (int64_t)nocc * nvir; g2.batch = naux;
        RT_TRY(gemm_f64(g2, stream));
    }
    if (K) {
        GemmF64 g3;
        g3.opa = 'N'; g3.opb = 'T'; g3.m = nb; g3.n = nb; g3.k = per / nb * naux;
        g3.A = X; g3.lda = nb; g3.B = X; g3.ldb = nb;
        g3.C = K; g3.rsC = 1; g3.csC = nb;
        const int64_t tiles = ceil_div(nb, BM) * ceil_div(nb, BN);
        const int64_t want = (4 * sm_count() + tiles - 1) / tiles;
        g3.splitk = (int)std::max<int64_t>(1, std::min<int64_t>(want, g3.k / 256));
        RT_TRY(gemm_f64(g3, stream));
    }
    return RT_OK;
}

}  // namespace rt

// ---------------------------------------------------------------------------
// Allocation-free float64 ov transform + RI-K.
//
// For callers that cannot allocate device memory while they run: hosts that
// hand the GPU's memory to a fixed arena managed by another runtime, or
// deployments where any cudaMalloc/cudaFree (with its implicit device
// synchronisation) is forbidden on the serving path.  The half-
// transform X^P = B^P C_occ lives in a fixed file-scope device array instead
// of scratch from the memory pool, and the aux slabs stream through it in
// blocks; K accumulates across blocks with beta = 1.  Nothing in the array
// needs to start at zero (every block's X is fully written before it is
// read).  Every call shares the array, so calls whose kernels overlap on the
// GPU (different streams, or different host threads) race on it.
// ---------------------------------------------------------------------------

namespace rt {
namespace {

constexpr size_t kNoAllocScratchDoubles = (size_t)4 << 20;  // 32 MiB
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

// Device address of the array, looked up once per device.
rt_status noalloc_scratch_address(double** out) {
    static std::mutex mu;
    static double* addr[64] = {};
    int dev = 0;
    RT_CUDA_TRY(cudaGetDevice(&dev));
    RT_REQUIRE(dev >= 0 && dev < 64, "rt_ri_ov_k_fp64_noalloc: device ordinal %d out of range", dev);
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        double* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
        if (e != cudaSuccess || p == nullptr) {
            set_error(RT_ERR_CUDA, "rt_ri_ov_k_fp64_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return RT_ERR_CUDA;
        }
        addr[dev] = p;
    }
    *out = addr[dev];
    return RT_OK;
}

// One dgemm_tile_kernel launch without split-K partials or profiling events.
rt_status launch_dgemm_noalloc(const GemmF64& q, cudaStream_t stream) {
    if (q.m == 0 || q.n == 0 || q.batch == 0) return RT_OK;
    GemmArgs g{};
    g.m = q.m; g.n = q.n; g.k = q.k; g.alpha = q.alpha; g.beta = q.beta;
    g.A = q.A; g.lda = q.lda; g.sA = q.sA; g.B = q.B; g.ldb = q.ldb; g.sB = q.sB;
    g.C = q.C; g.rsC = q.rsC; g.csC = q.csC; g.bsC = q.bsC; g.batch = q.batch;
    g.a_div = q.a_div; g.a_s1 = q.a_s1; g.c_md = q.c_md; g.c_ms1 = q.c_ms1;
    const int shape = pick_shape(q.m, q.n);
    g.tiles_m = ceil_div(q.m, (int64_t)tile_bm(shape));
    g.tiles_n = ceil_div(q.n, (int64_t)tile_bn(shape));
    g.splitk = 1;
    g.kchunk = ceil_div(std::max<int64_t>(q.k, 1), BK) * BK;
    if (q.k == 0) {
        scale_kernel<<<1024, 256, 0, stream>>>(g);
        return check_launch("scale_kernel");
    }
    dim3 grid((unsigned)(g.tiles_m * g.tiles_n), (unsigned)(q.batch < 65535 ? q.batch : 65535), 1u);
    const bool ta = q.opa == 'T', tb = q.opb == 'T';
    switch (shape) {
        case 1: launch_tile<1>(ta, tb, grid, g, stream); break;
        case 2: launch_tile<2>(ta, tb, grid, g, stream); break;
        case 3: launch_tile<3>(ta, tb, grid, g, stream); break;
        case 4: launch_tile<4>(ta, tb, grid, g, stream); break;
        default: launch_tile<0>(ta, tb, grid, g, stream); break;
    }
    return check_launch("dgemm_tile_kernel");
}

}  // namespace
}  // namespace rt

extern "C" rt_status rt_ri_ov_k_fp64_noalloc(const double* C, const double* B, int nb, int naux, int nocc, int nvir,
                                             double* ov, double* K, void* stream) {
    using namespace rt;
    RT_REQUIRE(nb >= 0 && naux >= 0 && nocc >= 0 && nvir >= 0, "rt_ri_ov_k_fp64_noalloc: negative dimension");
    const int64_t per = (int64_t)nb * nocc;
    RT_REQUIRE((size_t)per <= kNoAllocScratchDoubles,
               "rt_ri_ov_k_fp64_noalloc: nb*nocc = %lld exceeds the fixed scratch of %zu doubles (32 MiB)",
               (long long)per, kNoAllocScratchDoubles);
    cudaStream_t s = (cudaStream_t)stream;
    if (K && nb > 0 && (nocc == 0 || naux == 0))
        RT_CUDA_TRY(cudaMemsetAsync(K, 0, sizeof(double) * nb * (size_t)nb, s));
    if (per * naux == 0) {
        if (ov && (int64_t)nocc * nvir * naux > 0)
            RT_CUDA_TRY(cudaMemsetAsync(ov, 0, sizeof(double) * (size_t)nocc * nvir * naux, s));
        return RT_OK;
    }
    RT_REQUIRE(C && B, "rt_ri_ov_k_fp64_noalloc: null input pointer");
    double* X = nullptr;
    RT_TRY(noalloc_scratch_address(&X));
    const int64_t blk = std::min<int64_t>(naux, (int64_t)(kNoAllocScratchDoubles / (size_t)per));
    for (int64_t P0 = 0; P0 < naux; P0 += blk) {
        const int64_t np = std::min<int64_t>(blk, naux - P0);
        GemmF64 g1;
        g1.opa = 'N'; g1.opb = 'N'; g1.m = nb; g1.n = nocc; g1.k = nb;
        g1.A = B + P0 * (int64_t)nb * nb; g1.lda = nb; g1.sA = (int64_t)nb * nb;
        g1.B = C; g1.ldb = nb; g1.sB = 0;
        g1.C = X; g1.rsC = 1; g1.csC = nb; g1.bsC = per; g1.batch = np;
        RT_TRY(launch_dgemm_noalloc(g1, s));
        if (ov && nvir > 0) {
            GemmF64 g2;
            g2.opa = 'T'; g2.opb = 'N'; g2.m = nocc; g2.n = nvir; g2.k = nb;
            g2.A = X; g2.lda = nb; g2.sA = per;
            g2.B = C + per; g2.ldb = nb; g2.sB = 0;
            g2.C = ov + P0 * (int64_t)nocc * nvir; g2.rsC = 1; g2.csC = nocc; g2.bsC = (int64_t)nocc * nvir;
            g2.batch = np;
            RT_TRY(launch_dgemm_noalloc(g2, s));
        }
        if (K) {
            GemmF64 g3;
            g3.opa = 'N'; g3.opb = 'T'; g3.m = nb; g3.n = nb; g3.k = np * nocc;
            g3.A = X; g3.lda = nb; g3.B = X; g3.ldb = nb;
            g3.C = K; g3.rsC = 1; g3.csC = nb;
            g3.beta = P0 == 0 ? 0.0 : 1.0;
            RT_TRY(launch_dgemm_noalloc(g3, s));
        }
    }
    return RT_OK;
}
