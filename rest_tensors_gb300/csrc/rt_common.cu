// rt_common.cu - status text, per-thread error messages, the device error
// word, and stream-ordered scratch allocation.
#include <stdarg.h>
#include <stdlib.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <mutex>
#include <vector>

#include "rt_internal.cuh"

namespace rt {

static thread_local rt_status g_last_status = RT_OK;
static thread_local char g_last_msg[512] = "";

void set_error(rt_status s, const char* fmt, ...) {
    g_last_status = s;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_msg, sizeof(g_last_msg), fmt, ap);
    va_end(ap);
}

rt_status last_status() { return g_last_status; }

static std::atomic<long long> g_launches{0};

rt_status check_launch(const char* what) {
    g_launches.fetch_add(1, std::memory_order_relaxed);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(RT_ERR_CUDA, "launch of %s failed: %s", what, cudaGetErrorString(e));
        return RT_ERR_CUDA;
    }
    return RT_OK;
}

// Device error word: kernels OR flags into it (non-finite input, exhausted
// bounded waits).  One word per device; it is read and cleared by
// rt_sync_status() and by the host-pointer entry points.
__device__ unsigned int g_device_error_word;

unsigned int* error_word_device() {
    unsigned int* p = nullptr;
    if (cudaGetSymbolAddress((void**)&p, g_device_error_word) != cudaSuccess) return nullptr;
    return p;
}

rt_status error_word_check(cudaStream_t stream, const char* what) {
    unsigned int* p = error_word_device();
    if (!p) {
        set_error(RT_ERR_CUDA, "cannot locate the device error word");
        return RT_ERR_CUDA;
    }
    unsigned int h = 0;
    RT_CUDA_TRY(cudaMemcpyAsync(&h, p, sizeof(h), cudaMemcpyDeviceToHost, stream));
    RT_CUDA_TRY(cudaStreamSynchronize(stream));
    if (h) {
        RT_CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(unsigned int), stream));
        RT_CUDA_TRY(cudaStreamSynchronize(stream));
        if (h & DEV_ERR_ASYMMETRIC) {
            set_error(RT_ERR_INVALID_ARG, "%s: an input that must be symmetric is not (sampled check)", what);
            return RT_ERR_INVALID_ARG;
        }
        if (h & DEV_ERR_TIMEOUT) {
            set_error(RT_ERR_TIMEOUT, "%s: a device-side wait ran out of its cycle budget", what);
            return RT_ERR_TIMEOUT;
        }
        set_error(RT_ERR_NONFINITE, "%s: the split form received a non-finite input value", what);
        return RT_ERR_NONFINITE;
    }
    return RT_OK;
}

bool symmetry_check_enabled() {
    static const bool on = [] {
        const char* v = getenv("RT_CHECK_SYMMETRY");
        return v && v[0] && v[0] != '0';
    }();
    return on;
}

// Mirror pair t of slab P: a pseudo-random (mu, nu) with mu < nu, the same on
// host and device.
__host__ __device__ inline void sample_pair(int nb, int64_t P, int t, int& mu, int& nu) {
    uint64_t h = (uint64_t)P * 0x9E3779B97F4A7C15ull + (uint64_t)t * 0xBF58476D1CE4E5B9ull + 1;
    h ^= h >> 31;
    h *= 0x94D049BB133111EBull;
    h ^= h >> 29;
    const int a = (int)(h % (uint64_t)nb), b = (int)((h >> 32) % (uint64_t)nb);
    mu = a < b ? a : b;
    nu = a < b ? b : a;
}

__host__ __device__ inline bool mirror_equal(double x, double y) {
    const double d = x - y;
    return fabs(d) <= 1e-12 * (fabs(x) + fabs(y)) || (x == y);
}

// Every mirror pair of slab 0, then 64 sampled pairs of each slab.
__global__ void symmetry_sample_kernel(const double* __restrict__ B, int nb, int64_t nslab, unsigned int* err) {
    const int64_t n2 = (int64_t)nb * nb;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n2; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t mu = e % nb, nu = e / nb;
        if (mu < nu && !mirror_equal(B[e], B[nu + (int64_t)nb * mu])) atomicOr(err, DEV_ERR_ASYMMETRIC);
    }
    for (int64_t P = blockIdx.x; P < nslab; P += gridDim.x) {
        int mu, nu;
        sample_pair(nb, P, threadIdx.x, mu, nu);
        const double* b = B + P * n2;
        if (!mirror_equal(b[mu + (int64_t)nb * nu], b[nu + (int64_t)nb * mu])) atomicOr(err, DEV_ERR_ASYMMETRIC);
    }
}

rt_status symmetry_sample(const double* B, int nb, int64_t nslab, cudaStream_t stream) {
    if (nb < 2 || nslab <= 0) return RT_OK;
    unsigned int* err = error_word_device();
    RT_REQUIRE(err != nullptr, "cannot locate the device error word");
    symmetry_sample_kernel<<<(unsigned)std::min<int64_t>(nslab, 4 * sm_count()), 64, 0, stream>>>(B, nb, nslab, err);
    return check_launch("symmetry_sample_kernel");
}

rt_status symmetry_sample_host(const double* B, int nb, int64_t nslab, const char* what) {
    const int64_t n2 = (int64_t)nb * nb;
    for (int nu = 1; nslab > 0 && nu < nb; ++nu)
        for (int mu = 0; mu < nu; ++mu)
            if (!mirror_equal(B[mu + (int64_t)nb * nu], B[nu + (int64_t)nb * mu])) {
                set_error(RT_ERR_INVALID_ARG, "%s: slab 0 is not symmetric at (%d, %d)", what, mu, nu);
                return RT_ERR_INVALID_ARG;
            }
    for (int64_t P = 0; nb >= 2 && P < nslab; ++P)
        for (int t = 0; t < 64; ++t) {
            int mu, nu;
            sample_pair(nb, P, t, mu, nu);
            const double* b = B + P * n2;
            if (!mirror_equal(b[mu + (int64_t)nb * nu], b[nu + (int64_t)nb * mu])) {
                set_error(RT_ERR_INVALID_ARG, "%s: slab %lld is not symmetric at (%d, %d) (sampled check)", what,
                          (long long)P, mu, nu);
                return RT_ERR_INVALID_ARG;
            }
        }
    return RT_OK;
}

rt_status error_word_reset(cudaStream_t stream) {
    unsigned int* p = error_word_device();
    if (!p) {
        set_error(RT_ERR_CUDA, "cannot locate the device error word");
        return RT_ERR_CUDA;
    }
    RT_CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(unsigned int), stream));
    return RT_OK;
}

int sm_count() {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 148;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
    return n;
}

// ---------------------------------------------------------------- profiler --
namespace {
struct ProfRec {
    int kind;
    cudaEvent_t a, b;
    double flops;
};
std::mutex g_prof_mu;
std::atomic<bool> g_prof_on{false};
std::vector<ProfRec> g_prof_recs;
thread_local cudaEvent_t g_prof_pending[PROF_NKINDS] = {};
}  // namespace

bool prof_enabled() { return g_prof_on.load(std::memory_order_relaxed); }

void prof_begin(int kind, cudaStream_t s) {
    if (!prof_enabled()) return;
    cudaEvent_t a;
    if (cudaEventCreate(&a) != cudaSuccess) return;
    cudaEventRecord(a, s);
    g_prof_pending[kind] = a;
}

void prof_end(int kind, cudaStream_t s, double flops) {
    if (!prof_enabled() || !g_prof_pending[kind]) return;
    cudaEvent_t b;
    if (cudaEventCreate(&b) != cudaSuccess) return;
    cudaEventRecord(b, s);
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof_recs.push_back(ProfRec{kind, g_prof_pending[kind], b, flops});
    g_prof_pending[kind] = nullptr;
}

}  // namespace rt

extern "C" {

long long rt_launch_count(void) { return rt::g_launches.load(); }

void rt_profile_enable(int on) {
    std::lock_guard<std::mutex> lk(rt::g_prof_mu);
    for (auto& r : rt::g_prof_recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    rt::g_prof_recs.clear();
    rt::g_prof_on.store(on != 0);
}

rt_status rt_profile_get(int kind, double* total_ms, long long* launches, double* flops) {
    std::lock_guard<std::mutex> lk(rt::g_prof_mu);
    double ms = 0.0, fl = 0.0;
    long long n = 0;
    for (auto& r : rt::g_prof_recs) {
        if (r.kind != kind) continue;
        RT_CUDA_TRY(cudaEventSynchronize(r.b));
        float t = 0.f;
        RT_CUDA_TRY(cudaEventElapsedTime(&t, r.a, r.b));
        ms += t;
        fl += r.flops;
        ++n;
    }
    if (total_ms) *total_ms = ms;
    if (launches) *launches = n;
    if (flops) *flops = fl;
    return RT_OK;
}

int rt_version(void) { return (1 << 16) | 0; }

const char* rt_status_string(rt_status s) {
    switch (s) {
        case RT_OK: return "ok";
        case RT_ERR_INVALID_ARG: return "invalid argument";
        case RT_ERR_CUDA: return "CUDA error";
        case RT_ERR_NO_MEMORY: return "out of device memory";
        case RT_ERR_UNSUPPORTED: return "unsupported configuration";
        case RT_ERR_NONFINITE: return "non-finite input";
        case RT_ERR_TIMEOUT: return "device-side wait timed out";
        case RT_ERR_NOT_CONVERGED: return "not converged";
        default: return "unknown status";
    }
}

rt_status rt_last_status(void) { return rt::g_last_status; }
const char* rt_last_error(void) { return rt::g_last_msg; }

rt_status rt_sync_status(void* stream) {
    return rt::error_word_check((cudaStream_t)stream, "device kernels");
}

}  // extern "C"

namespace rt {

// Fault-injection hook for tests: when >= 0, the count of scratch allocations
// that still succeed; the next one fails with RT_ERR_NO_MEMORY.
static std::atomic<long long> g_fail_alloc_after{-1};

rt_status scratch_alloc(ScratchBuf& b, size_t bytes, cudaStream_t stream) {
    long long left = g_fail_alloc_after.load(std::memory_order_relaxed);
    while (left >= 0 && !g_fail_alloc_after.compare_exchange_weak(left, left - 1)) {
    }
    if (left == 0) {
        b.p = nullptr;
        set_error(RT_ERR_NO_MEMORY, "scratch allocation of %zu bytes failed: injected by rt_debug_fail_alloc_after",
                  bytes);
        return RT_ERR_NO_MEMORY;
    }
    static std::once_flag once;
    std::call_once(once, [] {
        // Keep freed pool memory mapped between calls so repeated calls do
        // not pay for re-mapping.
        int dev = 0;
        cudaGetDevice(&dev);
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t thr = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    });
    b.s = stream;
    if (bytes == 0) bytes = 256;
    cudaError_t e = cudaMallocAsync(&b.p, bytes, stream);
    if (e != cudaSuccess) {
        b.p = nullptr;
        cudaGetLastError();
        set_error(RT_ERR_NO_MEMORY, "scratch allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return RT_ERR_NO_MEMORY;
    }
    return RT_OK;
}

}  // namespace rt

namespace {

// One thread waits on an mbarrier that nothing arrives at, for at most
// `cycles` clock cycles, then records DEV_ERR_TIMEOUT and returns: the same
// bounded wait every pipeline of this library uses, run out on purpose.
__global__ void wait_timeout_kernel(long long cycles, unsigned int* err) {
    __shared__ uint64_t bar;
    const uint32_t a = (uint32_t)__cvta_generic_to_shared(&bar);
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(a) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    const long long t0 = clock64();
    while (true) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a)
            : "memory");
        if (ok) return;  // cannot happen: nothing arrives
        if (clock64() - t0 > cycles) {
            atomicOr(err, rt::DEV_ERR_TIMEOUT);
            return;
        }
    }
}

}  // namespace

extern "C" rt_status rt_debug_fail_alloc_after(long long n) {
    rt::g_fail_alloc_after.store(n < 0 ? -1 : n);
    return RT_OK;
}

extern "C" rt_status rt_debug_wait_timeout(long long cycles, void* stream) {
    RT_REQUIRE(cycles >= 0 && cycles <= 2000000000LL, "rt_debug_wait_timeout: cycles must be in [0, 2e9]");
    unsigned int* err = rt::error_word_device();
    RT_REQUIRE(err != nullptr, "rt_debug_wait_timeout: device error word unavailable");
    wait_timeout_kernel<<<1, 1, 0, (cudaStream_t)stream>>>(cycles, err);
    return rt::check_launch("wait_timeout_kernel");
}
