/*
 * rt_synth.h - deterministic synthetic inputs for the dense RI path.
 *
 * One definition, compiled for both the host (C/C++) and the device (CUDA),
 * so a three-centre tensor of any size can be generated in place on the GPU
 * and the same formula reproduced on the CPU.
 *
 *   ri3ao B[mu + nb*nu + nb*nb*P] = g(seed, P, min(mu,nu), max(mu,nu)) * exp(-|mu-nu|/20)
 *
 * g ~ N(0,1) is drawn with the Box-Muller transform (Box & Muller, 1958) from
 * two uniforms produced by the SplitMix64 mixing function (Steele, Lea &
 * Flood, 2014) applied to a counter built from (seed, P, lo, hi).  Keying on
 * the unordered pair makes every slab B^P exactly symmetric in (mu, nu), the
 * property the reference's RIFull ri3fn tensors carry (src/ri.rs:19-24 is the
 * container; src/external_libs/restmatr.f90:109-110 names the V^-1/2
 * contracted ri3fn producer).
 *
 * The library's log/sqrt/cos are used as-is.  Host libm and CUDA's device
 * functions may differ in the last bit, so bit-identical inputs on both sides
 * are obtained by generating on one side and copying.
 */
#ifndef RT_SYNTH_H
#define RT_SYNTH_H

#include <stdint.h>
#include <math.h>

#if defined(__CUDACC__)
#define RT_SYNTH_FN static __host__ __device__ __forceinline__
#else
#define RT_SYNTH_FN static inline
#endif

/* SplitMix64 output function: a published 64-bit bijective mixer. */
RT_SYNTH_FN uint64_t rt_splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

/* Uniform in (0, 1]: 53 random bits, offset by one ulp so log() is finite. */
RT_SYNTH_FN double rt_u01(uint64_t bits) {
    return ((double)(bits >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

/* N(0,1) sample for the counter (seed, a, b, c). */
RT_SYNTH_FN double rt_normal(uint64_t seed, uint64_t a, uint64_t b, uint64_t c) {
    uint64_t k = rt_splitmix64(seed ^ rt_splitmix64(a ^ rt_splitmix64((b << 32) ^ c)));
    uint64_t r1 = rt_splitmix64(k);
    uint64_t r2 = rt_splitmix64(k ^ 0xD1B54A32D192ED03ull);
    double u1 = rt_u01(r1);
    double u2 = rt_u01(r2);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* One element of the synthetic ri3ao tensor. */
RT_SYNTH_FN double rt_ri3ao_elem(uint64_t seed, int64_t P, int64_t mu, int64_t nu) {
    int64_t lo = mu < nu ? mu : nu;
    int64_t hi = mu < nu ? nu : mu;
    double g = rt_normal(seed, (uint64_t)P, (uint64_t)lo, (uint64_t)hi);
    return g * exp(-(double)(hi - lo) / 20.0);
}

/* One N(0,1) entry of the matrix whose QR factor gives the orbital coefficients. */
RT_SYNTH_FN double rt_coef_seed_elem(uint64_t seed, int64_t row, int64_t col) {
    return rt_normal(seed + 1u, 0x436F6566ull /* "Coef" */, (uint64_t)row, (uint64_t)col);
}

/* Orbital-energy-difference diagonal for the response problem, U[0.5, 3.0]. */
RT_SYNTH_FN double rt_delta_elem(uint64_t seed, int64_t ia) {
    uint64_t k = rt_splitmix64(seed ^ rt_splitmix64(0x44656C74ull ^ rt_splitmix64((uint64_t)ia)));
    /* fused multiply-add: one rounding, the same on the host and the device */
    return fma(2.5, rt_u01(k) - 0x1p-53, 0.5);
}

#endif /* RT_SYNTH_H */
