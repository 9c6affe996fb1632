// layout.cu - RIFull / MatrixFull layout utilities on the device.
//
// The reference moves blocks between its column-major containers with the
// Fortran copy routines (src/external_libs/restmatr.f90:197-285: copy_mm,
// copy_mr, copy_rm, copy_rr), permutes rank-3 tensors with the RIFull
// transposes (src/ri.rs:225-295) and packs the (mu, nu) pair index of a
// symmetric tensor with rifull_to_matfull_symm (src/ri.rs:296-307,
// richunk_reduce_by_symm at :330-341).  Every one of these is a strided
// gather/scatter of float64 elements, so they share one device primitive,
// strided_copy3, with two kernels:
//
//  * copy_rows_kernel: the output's unit-stride axis is also the input's
//    (or neither side has one): threads run along that axis, both sides
//    coalesced;
//  * copy_transpose_kernel: the axes differ; 32 x 32 tiles go through shared
//    memory so that reads run along the input's unit-stride axis and writes
//    along the output's.
//
// All of it is HBM-bound byte movement: 16 bytes of traffic per element.
#include <string.h>

#include <algorithm>

#include "rt_internal.cuh"

namespace rt {

namespace {

// Rows of the copied axis u; the two other axes are flattened into rows
// r = a1 + n1 a2.  Each thread moves four elements of a row (u, u + tx, ...)
// per visit, loads before stores, and walks its rows with an incremental
// (a1, a2) so that no division sits in the loop.  blockDim.x = 256 = tx * ty.
__global__ void __launch_bounds__(256) copy_rows_kernel(const double* __restrict__ in, double* __restrict__ out,
                                                        int64_t nu, int64_t isu, int64_t osu, int64_t n1,
                                                        int64_t is1, int64_t os1, int64_t n2, int64_t is2,
                                                        int64_t os2, int tx_log2, int64_t step_q, int64_t step_r) {
    const int tx = 1 << tx_log2, ty = 256 >> tx_log2;
    const int lx = threadIdx.x & (tx - 1), ly = threadIdx.x >> tx_log2;
    const int64_t r0 = (int64_t)blockIdx.y * ty + ly;
    int64_t a1 = r0 % n1, a2 = r0 / n1;
    const int64_t ustep = (int64_t)gridDim.x * tx * 4;
    for (; a2 < n2;) {
        const double* src = in + a1 * is1 + a2 * is2;
        double* dst = out + a1 * os1 + a2 * os2;
        for (int64_t u0 = (int64_t)blockIdx.x * tx * 4 + lx; u0 < nu; u0 += ustep) {
            double v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t u = u0 + (int64_t)q * tx;
                if (u < nu) v[q] = src[u * isu];
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int64_t u = u0 + (int64_t)q * tx;
                if (u < nu) dst[u * osu] = v[q];
            }
        }
        // next row: r += gridDim.y * ty, i.e. (a1, a2) += (step_r, step_q) with carry
        a1 += step_r;
        a2 += step_q;
        if (a1 >= n1) { a1 -= n1; ++a2; }
    }
}

// 32 x 32 tiles through shared memory, software-pipelined: a block loads
// its next tile into registers while it stores the current one, and the two
// shared-memory buffers alternate, so one barrier per tile suffices.
// 256 threads = 32 x 8; each thread holds four elements of a tile.
__global__ void __launch_bounds__(256) copy_transpose_kernel(const double* __restrict__ in,
                                                             double* __restrict__ out, int64_t nu, int64_t isu,
                                                             int64_t osu, int64_t nv, int64_t isv, int64_t osv,
                                                             int64_t nw, int64_t isw, int64_t osw) {
    // u: the output's unit-stride axis; v: the input's; w: the rest.
    __shared__ double tile[2][32][33];
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
    const int64_t tu = (nu + 31) / 32, tv = (nv + 31) / 32;
    const int64_t ntiles = tu * tv * nw;
    double r[4];
    auto load = [&](int64_t t) {
        const int64_t w = t / (tu * tv), rem = t % (tu * tv);
        const int64_t u0 = (rem % tu) * 32, v0 = (rem / tu) * 32;
        const double* src = in + w * isw;
#pragma unroll
        for (int q = 0; q < 4; ++q) {  // read along v
            const int64_t u = u0 + ty + 8 * q, v = v0 + tx;
            r[q] = (u < nu && v < nv) ? src[u * isu + v * isv] : 0.0;
        }
    };
    int64_t t = blockIdx.x;
    if (t < ntiles) load(t);
    int buf = 0;
    for (; t < ntiles; t += gridDim.x) {
#pragma unroll
        for (int q = 0; q < 4; ++q) tile[buf][ty + 8 * q][tx] = r[q];
        __syncthreads();
        const int64_t tn = t + gridDim.x;
        if (tn < ntiles) load(tn);  // in flight during the stores below
        const int64_t w = t / (tu * tv), rem = t % (tu * tv);
        const int64_t u0 = (rem % tu) * 32, v0 = (rem / tu) * 32;
        double* dst = out + w * osw;
#pragma unroll
        for (int q = 0; q < 4; ++q) {  // write along u
            const int64_t u = u0 + tx, v = v0 + ty + 8 * q;
            if (u < nu && v < nv) dst[u * osu + v * osv] = tile[buf][tx][ty + 8 * q];
        }
        buf ^= 1;
    }
}

// Upper triangle (row <= column) of every [nao, nao] slab, packed column by
// column: out[c (c + 1) / 2 + r + P npair] = in[r + c nao + P nao^2].
__global__ void __launch_bounds__(256) pack_upper_kernel(const double* __restrict__ in, double* __restrict__ out,
                                                         int nao, int64_t naux) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int c = blockIdx.x * 8 + warp;
    if (c >= nao) return;
    const int64_t npair = (int64_t)nao * (nao + 1) / 2;
    const int64_t colbase = (int64_t)c * (c + 1) / 2;
    for (int64_t P = blockIdx.y; P < naux; P += gridDim.y) {
        const double* src = in + P * nao * nao + (int64_t)c * nao;
        double* dst = out + P * npair + colbase;
        for (int r = lane; r <= c; r += 32) dst[r] = src[r];
    }
}

// Lowest and one-past-highest element offsets a strided block touches.
void block_span(const Copy3& c, bool output, int64_t& lo, int64_t& hi) {
    lo = 0;
    hi = 1;
    for (int d = 0; d < 3; ++d) {
        const int64_t s = output ? c.os[d] : c.is[d];
        const int64_t ext = (c.n[d] - 1) * s;
        if (ext < 0) lo += ext; else hi += ext;
    }
}

}  // namespace

rt_status strided_copy3(const double* in, double* out, const Copy3& c, cudaStream_t stream) {
    for (int d = 0; d < 3; ++d)
        if (c.n[d] <= 0) return RT_OK;
    int64_t n[3], is[3], os[3];
    for (int d = 0; d < 3; ++d) { n[d] = c.n[d]; is[d] = c.is[d]; os[d] = c.os[d]; }
    auto absl = [](int64_t x) { return x < 0 ? -x : x; };
    // u: smallest output stride among axes longer than 1; v: smallest input stride.
    int u = -1, v = -1;
    for (int d = 0; d < 3; ++d) {
        if (n[d] == 1) continue;
        if (u < 0 || absl(os[d]) < absl(os[u])) u = d;
        if (v < 0 || absl(is[d]) < absl(is[v])) v = d;
    }
    if (u < 0) u = v = 0;
    const int sms = sm_count();
    // Resident blocks per SM of a kernel, for grids that loop over their work.
    auto resident = [](const void* fn) {
        int nblk = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nblk, fn, 256, 0) != cudaSuccess || nblk < 1) nblk = 1;
        return nblk;
    };
    if (u == v || absl(is[v]) != 1 || absl(os[u]) != 1) {
        const int a = (u + 1) % 3, b = (u + 2) % 3;
        // Threads along u: the width (32..256, four elements each) that wastes the fewest lanes.
        int tx_log2 = 8;
        int64_t best = -1;
        for (int l = 8; l >= 5; --l) {
            const int64_t span = (int64_t)4 << l;
            const int64_t slots = (n[u] + span - 1) / span * span;
            if (best < 0 || slots < best) { best = slots; tx_log2 = l; }
        }
        const int tx = 1 << tx_log2, ty = 256 / tx;
        const int64_t nrow = n[a] * n[b];
        const int64_t gx = std::min<int64_t>((n[u] + 4 * tx - 1) / (4 * tx), 64);
        const int64_t gy = std::min<int64_t>(std::min<int64_t>((nrow + ty - 1) / ty, 65535),
                                             std::max<int64_t>(1, (int64_t)sms * resident((const void*)copy_rows_kernel) / gx));
        const int64_t S = gy * ty;  // rows advanced per visit
        copy_rows_kernel<<<dim3((unsigned)gx, (unsigned)gy), 256, 0, stream>>>(
            in, out, n[u], is[u], os[u], n[a], is[a], os[a], n[b], is[b], os[b], tx_log2, S / n[a], S % n[a]);
        return check_launch("copy_rows_kernel");
    }
    const int w = 3 - u - v;
    const int64_t ntiles = ((n[u] + 31) / 32) * ((n[v] + 31) / 32) * n[w];
    const int64_t grid = std::min<int64_t>(ntiles, (int64_t)sms * resident((const void*)copy_transpose_kernel));
    copy_transpose_kernel<<<(unsigned)grid, 256, 0, stream>>>(in, out, n[u], is[u], os[u], n[v], is[v], os[v],
                                                             n[w], is[w], os[w]);
    return check_launch("copy_transpose_kernel");
}

namespace {

// strided_copy3 with Fortran assignment semantics: if the source and
// destination blocks may share memory, the source is first gathered into
// scratch.
rt_status copy_block(const double* in, double* out, const Copy3& c, cudaStream_t stream) {
    for (int d = 0; d < 3; ++d)
        if (c.n[d] <= 0) return RT_OK;
    int64_t ilo, ihi, olo, ohi;
    block_span(c, false, ilo, ihi);
    block_span(c, true, olo, ohi);
    const bool overlap = (in + ilo < out + ohi) && (out + olo < in + ihi);
    if (!overlap) return strided_copy3(in, out, c, stream);
    const int64_t total = c.n[0] * c.n[1] * c.n[2];
    ScratchBuf tmp;
    RT_TRY(scratch_alloc(tmp, sizeof(double) * (size_t)total, stream));
    Copy3 g = c;
    g.os[0] = 1; g.os[1] = c.n[0]; g.os[2] = c.n[0] * c.n[1];
    RT_TRY(strided_copy3(in, tmp.as<double>(), g, stream));
    Copy3 p = c;
    p.is[0] = 1; p.is[1] = c.n[0]; p.is[2] = c.n[0] * c.n[1];
    return strided_copy3(tmp.as<double>(), out, p, stream);
}

bool in_range(int start, int len, int full) { return start >= 0 && len >= 0 && (int64_t)start + len <= full; }

}  // namespace

}  // namespace rt

using namespace rt;

extern "C" {

rt_status rt_copy_mm(int x_len, int y_len, const double* f_matr, int f_x_len, int f_y_len, int f_x_start,
                     int f_y_start, double* t_matr, int t_x_len, int t_y_len, int t_x_start, int t_y_start,
                     void* stream) {
    NvtxRange nvtx_range("rt_copy_mm");
    RT_REQUIRE(in_range(f_x_start, x_len, f_x_len) && in_range(f_y_start, y_len, f_y_len),
               "rt_copy_mm: source block outside the matrix");
    RT_REQUIRE(in_range(t_x_start, x_len, t_x_len) && in_range(t_y_start, y_len, t_y_len),
               "rt_copy_mm: target block outside the matrix");
    if ((int64_t)x_len * y_len == 0) return RT_OK;
    RT_REQUIRE(f_matr && t_matr, "rt_copy_mm: null pointer");
    Copy3 c;
    c.n[0] = x_len; c.n[1] = y_len; c.n[2] = 1;
    c.is[0] = 1; c.is[1] = f_x_len; c.is[2] = 0;
    c.os[0] = 1; c.os[1] = t_x_len; c.os[2] = 0;
    return copy_block(f_matr + f_x_start + (int64_t)f_y_start * f_x_len,
                      t_matr + t_x_start + (int64_t)t_y_start * t_x_len, c, (cudaStream_t)stream);
}

// Strides of the rank-3 tensor [X, Y, Z] along the two copied axes and the
// offset of the fixed index, by mode (restmatr.f90:227-235, 253-261):
//   mode 0: (a, b, x3)   mode 1: (a, x3, b)   mode 2: (x3, a, b)
static bool ri_mode_strides(int mode, int64_t X, int64_t Y, int64_t& sa, int64_t& sb, int64_t& sfix) {
    switch (mode) {
        case 0: sa = 1; sb = X; sfix = X * Y; return true;
        case 1: sa = 1; sb = X * Y; sfix = X; return true;
        case 2: sa = X; sb = X * Y; sfix = 1; return true;
        default: return false;
    }
}

static bool ri_mode_ranges(int mode, int a0, int alen, int b0, int blen, int fix, int X, int Y, int Z) {
    const int full[3] = {X, Y, Z};
    const int ax = mode == 2 ? 1 : 0, bx = mode == 0 ? 1 : 2, fx = mode == 0 ? 2 : (mode == 1 ? 1 : 0);
    return in_range(a0, alen, full[ax]) && in_range(b0, blen, full[bx]) && fix >= 0 && fix < full[fx];
}

rt_status rt_copy_mr(int x1_len, int x2_len, const double* f_matr, int f_x_len, int f_y_len, int f_x1_start,
                     int f_x2_start, double* t_ri, int t_x_len, int t_y_len, int t_z_len, int t_x1_start,
                     int t_x2_start, int t_x3, int mode, void* stream) {
    NvtxRange nvtx_range("rt_copy_mr");
    int64_t sa, sb, sfix;
    RT_REQUIRE(ri_mode_strides(mode, t_x_len, t_y_len, sa, sb, sfix), "rt_copy_mr: mode must be 0, 1 or 2");
    RT_REQUIRE(in_range(f_x1_start, x1_len, f_x_len) && in_range(f_x2_start, x2_len, f_y_len),
               "rt_copy_mr: source block outside the matrix");
    RT_REQUIRE(ri_mode_ranges(mode, t_x1_start, x1_len, t_x2_start, x2_len, t_x3, t_x_len, t_y_len, t_z_len),
               "rt_copy_mr: target block outside the tensor");
    if ((int64_t)x1_len * x2_len == 0) return RT_OK;
    RT_REQUIRE(f_matr && t_ri, "rt_copy_mr: null pointer");
    Copy3 c;
    c.n[0] = x1_len; c.n[1] = x2_len; c.n[2] = 1;
    c.is[0] = 1; c.is[1] = f_x_len; c.is[2] = 0;
    c.os[0] = sa; c.os[1] = sb; c.os[2] = 0;
    return copy_block(f_matr + f_x1_start + (int64_t)f_x2_start * f_x_len,
                      t_ri + t_x1_start * sa + t_x2_start * sb + t_x3 * sfix, c, (cudaStream_t)stream);
}

rt_status rt_copy_rm(int x1_len, int x2_len, const double* f_ri, int f_x_len, int f_y_len, int f_z_len,
                     int f_x1_start, int f_x2_start, int f_x3, int mode, double* t_matr, int t_x_len, int t_y_len,
                     int t_x1_start, int t_x2_start, void* stream) {
    NvtxRange nvtx_range("rt_copy_rm");
    int64_t sa, sb, sfix;
    RT_REQUIRE(ri_mode_strides(mode, f_x_len, f_y_len, sa, sb, sfix), "rt_copy_rm: mode must be 0, 1 or 2");
    RT_REQUIRE(ri_mode_ranges(mode, f_x1_start, x1_len, f_x2_start, x2_len, f_x3, f_x_len, f_y_len, f_z_len),
               "rt_copy_rm: source block outside the tensor");
    RT_REQUIRE(in_range(t_x1_start, x1_len, t_x_len) && in_range(t_x2_start, x2_len, t_y_len),
               "rt_copy_rm: target block outside the matrix");
    if ((int64_t)x1_len * x2_len == 0) return RT_OK;
    RT_REQUIRE(f_ri && t_matr, "rt_copy_rm: null pointer");
    Copy3 c;
    c.n[0] = x1_len; c.n[1] = x2_len; c.n[2] = 1;
    c.is[0] = sa; c.is[1] = sb; c.is[2] = 0;
    c.os[0] = 1; c.os[1] = t_x_len; c.os[2] = 0;
    return copy_block(f_ri + f_x1_start * sa + f_x2_start * sb + f_x3 * sfix,
                      t_matr + t_x1_start + (int64_t)t_x2_start * t_x_len, c, (cudaStream_t)stream);
}

rt_status rt_copy_rr(int x1_len, int x2_len, int x3_len, const double* f_ri, int f_x1_len, int f_x2_len,
                     int f_x3_len, int f_x1_start, int f_x2_start, int f_x3_start, double* t_ri, int t_x1_len,
                     int t_x2_len, int t_x3_len, int t_x1_start, int t_x2_start, int t_x3_start, void* stream) {
    NvtxRange nvtx_range("rt_copy_rr");
    RT_REQUIRE(in_range(f_x1_start, x1_len, f_x1_len) && in_range(f_x2_start, x2_len, f_x2_len) &&
                   in_range(f_x3_start, x3_len, f_x3_len),
               "rt_copy_rr: source block outside the tensor");
    RT_REQUIRE(in_range(t_x1_start, x1_len, t_x1_len) && in_range(t_x2_start, x2_len, t_x2_len) &&
                   in_range(t_x3_start, x3_len, t_x3_len),
               "rt_copy_rr: target block outside the tensor");
    if ((int64_t)x1_len * x2_len * x3_len == 0) return RT_OK;
    RT_REQUIRE(f_ri && t_ri, "rt_copy_rr: null pointer");
    const int64_t fxy = (int64_t)f_x1_len * f_x2_len, txy = (int64_t)t_x1_len * t_x2_len;
    Copy3 c;
    c.n[0] = x1_len; c.n[1] = x2_len; c.n[2] = x3_len;
    c.is[0] = 1; c.is[1] = f_x1_len; c.is[2] = fxy;
    c.os[0] = 1; c.os[1] = t_x1_len; c.os[2] = txy;
    return copy_block(f_ri + f_x1_start + (int64_t)f_x2_start * f_x1_len + f_x3_start * fxy,
                      t_ri + t_x1_start + (int64_t)t_x2_start * t_x1_len + t_x3_start * txy, c,
                      (cudaStream_t)stream);
}

rt_status rt_ri_transpose(const double* in, int i, int j, int k, const char* order, double* out, void* stream) {
    NvtxRange nvtx_range("rt_ri_transpose");
    RT_REQUIRE(i >= 0 && j >= 0 && k >= 0, "rt_ri_transpose: negative dimension");
    RT_REQUIRE(order && strlen(order) == 3, "rt_ri_transpose: order must name three axes");
    const int n_in[3] = {i, j, k};
    const int64_t s_in[3] = {1, (int64_t)i, (int64_t)i * j};
    int ax[3];
    bool seen[3] = {false, false, false};
    for (int d = 0; d < 3; ++d) {
        const char ch = order[d];
        RT_REQUIRE(ch == 'i' || ch == 'j' || ch == 'k', "rt_ri_transpose: order letters must be i, j, k");
        ax[d] = ch - 'i';
        RT_REQUIRE(!seen[ax[d]], "rt_ri_transpose: order repeats an axis");
        seen[ax[d]] = true;
    }
    if ((int64_t)i * j * k == 0) return RT_OK;
    RT_REQUIRE(in && out, "rt_ri_transpose: null pointer");
    // Output axis d runs over input axis ax[d]; output strides follow the output's own sizes.
    Copy3 c;
    int64_t os = 1;
    for (int d = 0; d < 3; ++d) {
        c.n[d] = n_in[ax[d]];
        c.is[d] = s_in[ax[d]];
        c.os[d] = os;
        os *= n_in[ax[d]];
    }
    return copy_block(in, out, c, (cudaStream_t)stream);
}

rt_status rt_ri_pack_symm(const double* in, int nao, int naux, double* out, void* stream) {
    NvtxRange nvtx_range("rt_ri_pack_symm");
    RT_REQUIRE(nao >= 0 && naux >= 0, "rt_ri_pack_symm: negative dimension");
    if ((int64_t)nao * naux == 0) return RT_OK;
    RT_REQUIRE(in && out, "rt_ri_pack_symm: null pointer");
    const int64_t npair = (int64_t)nao * (nao + 1) / 2;
    RT_REQUIRE(out + npair * naux <= in || in + (int64_t)nao * nao * naux <= out,
               "rt_ri_pack_symm: input and output overlap");
    const int gx = (nao + 7) / 8;
    const int64_t gy = std::min<int64_t>(naux, std::max<int64_t>(1, (int64_t)sm_count() * 32 / gx));
    pack_upper_kernel<<<dim3(gx, (unsigned)std::min<int64_t>(gy, 65535)), 256, 0, (cudaStream_t)stream>>>(
        in, out, nao, naux);
    return check_launch("pack_upper_kernel");
}

}  // extern "C"
