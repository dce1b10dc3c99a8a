/*
 * gbrt_rng.h -- the random stream of the path tracer, shared by the CUDA kernels,
 * host code and anything that wants to replay a path (matched random numbers).
 *
 * visionaray's schedulers seed a sequential engine per pixel (make_random_seed.h:23-37
 * + thrust / std minstd engines, random_generator.h:29-63), so its CPU and GPU
 * streams differ and a path cannot be replayed out of order.  Here draw k of sample s
 * of pixel p in frame f is a pure function of (f, p, s, k): a SplitMix64-finalised
 * hash (Steele, Lea & Flood 2014), top 24 bits scaled to [0, 1).  Integer arithmetic
 * only, so every host and device produces the same floats.  Any object with
 * `value_type` and `next()` drives visionaray's pathtracing::kernel (pathtracing.inl),
 * so the same stream also drives the reference.
 */
#ifndef VISIONARAY_GB300_GBRT_RNG_H
#define VISIONARAY_GB300_GBRT_RNG_H 1

#include <stdint.h>

#if defined(__CUDACC__)
#define GBRT_HD __host__ __device__ __forceinline__
#define GBRT_HD_MEMBER __host__ __device__ __forceinline__
#else
#define GBRT_HD static inline
#define GBRT_HD_MEMBER inline
#endif

GBRT_HD uint64_t gbrt_rng_mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Uniform float in [0, 1): draw `k` of sample `sample` of pixel `pixel`, frame `frame`. */
GBRT_HD float gbrt_rng_u01(uint32_t frame, uint32_t pixel, uint32_t sample, uint32_t k)
{
    uint64_t key = ((uint64_t)pixel << 32) | (uint64_t)sample;
    uint64_t h = gbrt_rng_mix64(gbrt_rng_mix64(key ^ ((uint64_t)(frame + 1u) * 0x9E3779B97F4A7C15ull)) +
                                (uint64_t)(k + 1u) * 0xD1B54A32D192ED03ull);
    return (float)(uint32_t)(h >> 40) * (1.0f / 16777216.0f);
}

#ifdef __cplusplus
/* A visionaray-style generator over that stream: value_type + next(). */
struct gbrt_sample_generator
{
    using value_type = float;
    uint32_t frame, pixel, sample, k;
    GBRT_HD_MEMBER float next() { return gbrt_rng_u01(frame, pixel, sample, k++); }
};
#endif

#endif
