// pyre_math.cuh — vector maths, sampler and hashing shared by host and device.
//
// Operation order follows the Pyre CPU path (glam 0.29 Vec3 semantics):
// dot = (x*x' + y*y') + z*z', cross = (y*z' - y'*z, ...), normalize = v * (1/|v|),
// f32::min/max ignore NaN (fminf/fmaxf). Every translation unit that includes
// this header is compiled without FMA contraction (nvcc --fmad=false,
// g++ -ffp-contract=off), so the kernels reproduce the reference's binary32
// rounding for +,-,*,/ and sqrt.
#pragma once
#include <cstdint>
#include <cmath>

#if defined(__CUDACC__)
#define PYRE_HD __host__ __device__ __forceinline__
#else
#define PYRE_HD inline
#endif

namespace pyre {

#define PYRE_PI 3.14159265358979323846f
#define PYRE_TAU 6.28318530717958647692f
#define PYRE_FRAC_PI_2 1.57079632679489661923f
#define PYRE_FRAC_PI_4 0.785398163397448309615f
#define PYRE_FRAC_1_PI 0.318309886183790671538f

struct f2 { float x, y; };
struct f3 {
    float x, y, z;
};
PYRE_HD f3 mk3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
PYRE_HD f3 splat3(float v) { return mk3(v, v, v); }
PYRE_HD f3 operator+(f3 a, f3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
PYRE_HD f3 operator-(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
PYRE_HD f3 operator-(f3 a) { return mk3(-a.x, -a.y, -a.z); }
PYRE_HD f3 operator*(f3 a, f3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
PYRE_HD f3 operator*(f3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
PYRE_HD f3 operator*(float s, f3 a) { return mk3(s * a.x, s * a.y, s * a.z); }
PYRE_HD f3 operator/(f3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
PYRE_HD bool is_zero3(f3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }
PYRE_HD bool eq3(f3 a, f3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
PYRE_HD float dot3(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PYRE_HD f3 cross3(f3 a, f3 b) { return mk3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y); }
PYRE_HD float len2(f3 a) { return dot3(a, a); }
PYRE_HD float len3(f3 a) { return sqrtf(dot3(a, a)); }
PYRE_HD f3 normalize3(f3 a) { float r = 1.0f / len3(a); return a * r; }
PYRE_HD bool finite_(float v) {
#if defined(__CUDACC__)
    return isfinite(v);
#else
    return std::isfinite(v);
#endif
}
PYRE_HD f3 normalize_or_zero3(f3 a) {
    float r = 1.0f / len3(a);
    if (finite_(r) && r > 0.0f) return a * r;
    return splat3(0.0f);
}
PYRE_HD f3 vmin3(f3 a, f3 b) { return mk3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
PYRE_HD f3 vmax3(f3 a, f3 b) { return mk3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
PYRE_HD float max_elem3(f3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
PYRE_HD float min_elem3(f3 a) { return fminf(a.x, fminf(a.y, a.z)); }
PYRE_HD f3 lerp3(f3 a, f3 b, float s) { return a * (1.0f - s) + b * s; }
// Rust f32::clamp: NaN passes through.
PYRE_HD float clampf_(float v, float lo, float hi) { if (v < lo) v = lo; if (v > hi) v = hi; return v; }
// f32::powi(x, 5) as LLVM expands it: x * ((x*x)*(x*x)).
PYRE_HD float powi5(float x) { float x2 = x * x; float x4 = x2 * x2; return x * x4; }

// ---------------------------------------------------------------------------
// Per-sample seed and sampler (crates/pyre/src/sampler.rs:15-49, with the
// published Xoshiro256++ / SplitMix64 algorithms of rand_xoshiro 0.7 and the
// 24-bit float conversion of rand 0.9).
// ---------------------------------------------------------------------------
PYRE_HD uint64_t pixel_seed(uint32_t x, uint32_t y, uint32_t sample) {
    uint64_t h = ((uint64_t)x << 32) | (uint64_t)y;
    h ^= (uint64_t)sample * 0x9E3779B97F4A7C15ull;
    h ^= h >> 30;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 27;
    h *= 0x94D049BB133111EBull;
    return h ^ (h >> 31);
}

PYRE_HD uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

struct Rng {
    uint64_t s0, s1, s2, s3;
    PYRE_HD void seed(uint64_t seed) {
        uint64_t x = seed;
        uint64_t st[4];
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
        for (int i = 0; i < 4; ++i) {
            x += 0x9E3779B97F4A7C15ull;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            st[i] = z ^ (z >> 31);
        }
        s0 = st[0]; s1 = st[1]; s2 = st[2]; s3 = st[3];
    }
    PYRE_HD uint64_t next_u64() {
        uint64_t result = rotl64(s0 + s3, 23) + s0;
        uint64_t t = s1 << 17;
        s2 ^= s0; s3 ^= s1; s1 ^= s2; s0 ^= s3;
        s2 ^= t; s3 = rotl64(s3, 45);
        return result;
    }
    PYRE_HD float next_f32() {
        uint32_t u = (uint32_t)(next_u64() >> 32);
        return (float)(u >> 8) * (1.0f / 16777216.0f);
    }
    PYRE_HD f2 next_vec2() { f2 v; v.x = next_f32(); v.y = next_f32(); return v; }
};

}  // namespace pyre
