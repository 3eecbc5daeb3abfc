// pyre_oracle.cpp — CPU ORACLE for the GB300 wavefront path tracer.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker, never the product:
// only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
// it. It restates, function by function, the CPU path of the Pyre renderer
// (Rust, crates/pyre) in C++17 with IEEE binary32 arithmetic, no FMA
// contraction (-ffp-contract=off) and no fast-math, so that its results can
// be compared with the CUDA kernels on identical inputs.
//
// Every function cites the reference file:line it follows (paths are
// relative to the Pyre repository root).
//
// Parity status
// -------------
// * Pinned by the reference's own unit tests (tests/golden/reference_kats.json):
//   Möller–Trumbore hit/miss/closest (crates/pyre/src/geometry/mesh.rs:197-234),
//   Distribution1D/2D (crates/pyre/src/distribution.rs:178-220), Disney
//   sample/eval/pdf self-consistency (crates/pyre/src/material.rs:332-387).
// * UNPINNED (no reference test or golden output exists, and the reference
//   cannot be built here: no Rust toolchain, crates not vendored):
//   - rand_xoshiro 0.7.0 `Xoshiro256PlusPlus::seed_from_u64` is assumed to be
//     "four successive SplitMix64 outputs (state += 0x9E3779B97F4A7C15,
//     xor-shift 30/27/31 finaliser) form s[0..3]" (published algorithm,
//     Blackman & Vigna); `next_u32` is assumed to be `next_u64() >> 32`.
//   - rand 0.9.4 `random::<f32>()` is assumed to be
//     `(next_u32() >> 8) as f32 * 2^-24` (24-bit multiply method).
//   - glam 0.29.3 operation order is assumed: dot = (x*x' + y*y') + z*z';
//     cross = (y*z' - y'*z, z*x' - z'*x, x*y' - x'*y); normalize = v * (1/sqrt(dot));
//     normalize_or_zero returns 0 unless 1/len is finite and > 0;
//     lerp(a, b, s) = a*(1-s) + b*s; Vec3::clamp = max then min.
//   - f32::powi(x, 5) is assumed to lower to x * ((x*x)*(x*x)) (LLVM's
//     repeated-squaring expansion of powi with a constant exponent).
//   - Transcendentals come from the platform libm (sinf, cosf, tanf, acosf,
//     atan2f), as Rust's std does on Linux.
//
// Additions that the reference does not have (reporting only):
//   * the closest hit also reports (instance, triangle, u, v);
//   * a "canonical" tie rule (min t, then lowest (instance, triangle)) that
//     makes hit identity independent of traversal order;
//   * FP64 accumulation of per-sample radiance for the high-spp oracle;
//   * pixel crops and sample ranges [spp_begin, spp_end).

#include <cmath>
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <vector>
#include <memory>
#include <algorithm>
#include <limits>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

static const float PI = 3.14159265358979323846f;
static const float TAU = 6.28318530717958647692f;
static const float FRAC_PI_2 = 1.57079632679489661923f;
static const float FRAC_PI_4 = 0.785398163397448309615f;
static const float FRAC_1_PI = 0.318309886183790671538f;
static const float INF = std::numeric_limits<float>::infinity();

// ---------------------------------------------------------------------------
// glam-equivalent vector maths (crates/pyre/src/math.rs relies on glam 0.29.3)
// ---------------------------------------------------------------------------
struct V2 { float x, y; };
struct V3 {
    float x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(float a, float b, float c) : x(a), y(b), z(c) {}
    static V3 splat(float v) { return V3(v, v, v); }
};
static inline V3 operator+(V3 a, V3 b) { return V3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 operator-(V3 a, V3 b) { return V3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 operator-(V3 a) { return V3(-a.x, -a.y, -a.z); }
static inline V3 operator*(V3 a, V3 b) { return V3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 operator*(V3 a, float s) { return V3(a.x * s, a.y * s, a.z * s); }
static inline V3 operator*(float s, V3 a) { return V3(s * a.x, s * a.y, s * a.z); }
static inline V3 operator/(V3 a, float s) { return V3(a.x / s, a.y / s, a.z / s); }
static inline V3 operator/(V3 a, V3 b) { return V3(a.x / b.x, a.y / b.y, a.z / b.z); }
static inline bool operator==(V3 a, V3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
static inline bool operator!=(V3 a, V3 b) { return !(a == b); }
static inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) {
    return V3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
static inline float length_squared(V3 a) { return dot(a, a); }
static inline float length(V3 a) { return std::sqrt(dot(a, a)); }
static inline V3 normalize(V3 a) { float r = 1.0f / length(a); return a * r; }
static inline V3 normalize_or_zero(V3 a) {
    float r = 1.0f / length(a);
    if (std::isfinite(r) && r > 0.0f) return a * r;
    return V3();
}
// Rust f32::min / f32::max ignore a NaN operand, like C fminf / fmaxf.
static inline float fmin_(float a, float b) { return std::fmin(a, b); }
static inline float fmax_(float a, float b) { return std::fmax(a, b); }
static inline V3 vmin(V3 a, V3 b) { return V3(fmin_(a.x, b.x), fmin_(a.y, b.y), fmin_(a.z, b.z)); }
static inline V3 vmax(V3 a, V3 b) { return V3(fmax_(a.x, b.x), fmax_(a.y, b.y), fmax_(a.z, b.z)); }
static inline float max_element(V3 a) { return fmax_(a.x, fmax_(a.y, a.z)); }
static inline float min_element(V3 a) { return fmin_(a.x, fmin_(a.y, a.z)); }
static inline V3 lerp(V3 a, V3 b, float s) { return a * (1.0f - s) + b * s; }
// Rust f32::clamp (std): NaN passes through.
static inline float clampf(float v, float lo, float hi) {
    if (v < lo) v = lo;
    if (v > hi) v = hi;
    return v;
}
static inline float powi5(float x) { float x2 = x * x; float x4 = x2 * x2; return x * x4; }

// ---------------------------------------------------------------------------
// Ray / Bounds / Frame — crates/pyre/src/math.rs:3-104
// ---------------------------------------------------------------------------
struct Ray {
    V3 origin, direction;
    float t_min, t_max, time;
    // Ray::new normalizes (math.rs:16-24).
    static Ray make(V3 o, V3 d) { Ray r; r.origin = o; r.direction = normalize(d); r.t_min = 1e-4f; r.t_max = INF; r.time = 0.0f; return r; }
    V3 at(float t) const { return origin + direction * t; }  // math.rs:26-28
};

struct Bounds3 {
    V3 min, max;
    static Bounds3 empty() { Bounds3 b; b.min = V3::splat(INF); b.max = V3::splat(-INF); return b; }
    static Bounds3 point(V3 p) { Bounds3 b; b.min = p; b.max = p; return b; }
    Bounds3 unite(const Bounds3& o) const { Bounds3 b; b.min = vmin(min, o.min); b.max = vmax(max, o.max); return b; }
    Bounds3 extend(V3 p) const { Bounds3 b; b.min = vmin(min, p); b.max = vmax(max, p); return b; }
    V3 diagonal() const { return max - min; }
    float surface_area() const { V3 d = diagonal(); return 2.0f * (d.x * d.y + d.x * d.z + d.y * d.z); }
};

struct Frame {  // math.rs:88-104
    V3 t, bt, n;
    static Frame from_normal(V3 n) {
        V3 helper = std::fabs(n.x) > 0.9f ? V3(0, 1, 0) : V3(1, 0, 0);
        Frame f; f.t = normalize(cross(helper, n)); f.bt = cross(n, f.t); f.n = n; return f;
    }
    V3 to_local(V3 v) const { return V3(dot(v, t), dot(v, bt), dot(v, n)); }
    V3 to_world(V3 v) const { return v.x * t + v.y * bt + v.z * n; }
};

// ---------------------------------------------------------------------------
// Sampler — crates/pyre/src/sampler.rs:15-49 (+ rand_xoshiro 0.7.0 / rand 0.9.4)
// ---------------------------------------------------------------------------
static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

struct Xoshiro256pp {
    uint64_t s[4];
    // seed_from_u64 via SplitMix64 (assumption recorded in the header).
    static Xoshiro256pp seed_from_u64(uint64_t seed) {
        Xoshiro256pp r;
        uint64_t x = seed;
        for (int i = 0; i < 4; ++i) {
            x += 0x9E3779B97F4A7C15ull;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            r.s[i] = z ^ (z >> 31);
        }
        return r;
    }
    uint64_t next_u64() {
        uint64_t result = rotl(s[0] + s[3], 23) + s[0];
        uint64_t t = s[1] << 17;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t; s[3] = rotl(s[3], 45);
        return result;
    }
    uint32_t next_u32() { return (uint32_t)(next_u64() >> 32); }
    float next_f32() { return (float)(next_u32() >> 8) * (1.0f / 16777216.0f); }
};

struct Sampler {  // IndependentSampler, sampler.rs:15-36
    Xoshiro256pp rng;
    explicit Sampler(uint64_t seed) : rng(Xoshiro256pp::seed_from_u64(seed)) {}
    float next_f32() { return rng.next_f32(); }
    V2 next_vec2() { V2 v; v.x = rng.next_f32(); v.y = rng.next_f32(); return v; }
};

static inline uint64_t pixel_seed(uint32_t x, uint32_t y, uint32_t sample) {  // sampler.rs:41-49
    uint64_t h = ((uint64_t)x << 32) | (uint64_t)y;
    h ^= (uint64_t)sample * 0x9E3779B97F4A7C15ull;
    h ^= h >> 30;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 27;
    h *= 0x94D049BB133111EBull;
    return h ^ (h >> 31);
}

// ---------------------------------------------------------------------------
// Distributions — crates/pyre/src/distribution.rs:12-172
// ---------------------------------------------------------------------------
static V2 concentric_disk(V2 u) {  // distribution.rs:12-23
    V2 off; off.x = 2.0f * u.x - 1.0f; off.y = 2.0f * u.y - 1.0f;
    if (off.x == 0.0f && off.y == 0.0f) { V2 z; z.x = 0; z.y = 0; return z; }
    float r, theta;
    if (std::fabs(off.x) > std::fabs(off.y)) { r = off.x; theta = FRAC_PI_4 * (off.y / off.x); }
    else { r = off.y; theta = FRAC_PI_2 - FRAC_PI_4 * (off.x / off.y); }
    V2 o; o.x = r * std::cos(theta); o.y = r * std::sin(theta); return o;
}

struct Distribution1D {  // distribution.rs:28-113
    std::vector<float> cdf;
    float integral = 0.0f;
    size_t n = 0;
    Distribution1D() {}
    explicit Distribution1D(const float* w, size_t count) {
        n = count;
        cdf.reserve(n + 1);
        cdf.push_back(0.0f);
        float acc = 0.0f;
        for (size_t i = 0; i < n; ++i) { acc += fmax_(w[i], 0.0f); cdf.push_back(acc); }
        integral = acc;
        if (integral > 0.0f) { for (auto& c : cdf) c /= integral; }
        else { for (size_t i = 0; i < cdf.size(); ++i) cdf[i] = (float)i / (float)n; }
    }
    // returns t, writes pdf and bin (distribution.rs:79-101)
    float sample_continuous(float u, float* pdf, size_t* bin_out) const {
        size_t lo = 1, hi = cdf.size() - 1;
        while (lo < hi) {
            size_t mid = (lo + hi) / 2;
            if (cdf[mid] <= u) lo = mid + 1; else hi = mid;
        }
        size_t bin = std::min(lo - 1, n - 1);
        float cdf_lo = cdf[bin], cdf_hi = cdf[bin + 1];
        float bin_size = fmax_(cdf_hi - cdf_lo, 1e-20f);
        float du = (u - cdf_lo) / bin_size;
        float t = ((float)bin + du) / (float)n;
        *pdf = bin_size * (float)n;
        *bin_out = bin;
        return t;
    }
    float pdf_at(float t) const {  // distribution.rs:104-112
        if (t < 0.0f || t >= 1.0f || n == 0) return 0.0f;
        size_t bin = std::min((size_t)(t * (float)n), n - 1);
        return (cdf[bin + 1] - cdf[bin]) * (float)n;
    }
};

struct Distribution2D {  // distribution.rs:119-172
    size_t width = 0, height = 0;
    std::vector<Distribution1D> conditionals;
    Distribution1D marginal;
    Distribution2D() {}
    Distribution2D(const float* w, size_t width_, size_t height_) : width(width_), height(height_) {
        std::vector<float> row_integrals;
        row_integrals.reserve(height);
        conditionals.reserve(height);
        for (size_t y = 0; y < height; ++y) {
            conditionals.emplace_back(w + y * width, width);
            row_integrals.push_back(conditionals.back().integral);
        }
        marginal = Distribution1D(row_integrals.data(), height);
    }
    V2 sample_continuous(V2 s, float* pdf) const {
        float pdf_v, pdf_u; size_t row, col;
        float v = marginal.sample_continuous(s.y, &pdf_v, &row);
        float u = conditionals[row].sample_continuous(s.x, &pdf_u, &col);
        *pdf = pdf_u * pdf_v;
        V2 o; o.x = u; o.y = v; return o;
    }
    float pdf_at(V2 uv) const {
        if (uv.x < 0.0f || uv.x >= 1.0f || uv.y < 0.0f || uv.y >= 1.0f) return 0.0f;
        size_t row = std::min((size_t)(uv.y * (float)height), height - 1);
        return conditionals[row].pdf_at(uv.x) * marginal.pdf_at(uv.y);
    }
};

// ---------------------------------------------------------------------------
// Camera — crates/pyre/src/camera.rs:28-143
// ---------------------------------------------------------------------------
struct Camera {
    int thin_lens = 0;
    V3 origin, forward, right, up;
    float half_width = 0, half_height = 0, aperture_radius = 0, focus_distance = 0;
    // look_at: camera.rs:49-72 / 105-122
    static Camera look_at(V3 origin, V3 target, V3 world_up, float vfov_deg, float aspect,
                          int thin, float aperture_radius, float focus_distance) {
        Camera c;
        c.thin_lens = thin;
        c.origin = origin;
        c.forward = normalize(target - origin);
        c.right = normalize(cross(c.forward, world_up));
        c.up = cross(c.right, c.forward);
        const float to_rad = PI / 180.0f;  // f32::to_radians
        c.half_height = std::tan(vfov_deg * to_rad / 2.0f);
        c.half_width = aspect * c.half_height;
        c.aperture_radius = aperture_radius;
        c.focus_distance = focus_distance;
        return c;
    }
    Ray generate_ray(V2 ndc, V2 lens, float time) const {
        if (!thin_lens) {  // camera.rs:65-73
            V3 d = forward + ndc.x * half_width * right + ndc.y * half_height * up;
            Ray r = Ray::make(origin, d); r.time = time; return r;
        }
        // camera.rs:125-143
        V3 pinhole_dir = normalize(forward + ndc.x * half_width * right + ndc.y * half_height * up);
        float focal_t = focus_distance / dot(pinhole_dir, forward);
        V3 focal_point = origin + focal_t * pinhole_dir;
        V2 disk = concentric_disk(lens);
        V3 lens_offset = aperture_radius * (disk.x * right + disk.y * up);
        V3 lens_origin = origin + lens_offset;
        V3 dir = normalize(focal_point - lens_origin);
        Ray r = Ray::make(lens_origin, dir); r.time = time; return r;
    }
};

// ---------------------------------------------------------------------------
// BVH — crates/pyre/src/geometry/bvh.rs:13-409
// ---------------------------------------------------------------------------
#pragma pack(push, 1)
struct BvhNode {  // bvh.rs:18-30 (field order and sizes; 32 bytes)
    float bmin[3], bmax[3];
    uint32_t offset;
    uint16_t n_primitives;
    uint8_t axis;
    uint8_t pad;
};
#pragma pack(pop)
static_assert(sizeof(BvhNode) == 32, "BvhNode is 32 bytes");

static const int BINS = 12;
static const size_t MAX_PRIMS_PER_LEAF = 8;
static const float TRAVERSAL_COST = 1.0f, INTERSECT_COST = 2.0f;

static inline float axis_value(V3 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
static inline int max_axis(V3 v) {  // bvh.rs:164-172
    if (v.x >= v.y && v.x >= v.z) return 0;
    if (v.y >= v.z) return 1;
    return 2;
}

struct BvhBuilder {
    std::vector<BvhNode>& nodes;
    uint32_t* indices;
    const Bounds3* pb;
    const V3* pc;

    uint32_t push_leaf(const Bounds3& b, uint32_t start, uint16_t n) {  // bvh.rs:348-358
        BvhNode nd; std::memset(&nd, 0, sizeof nd);
        nd.bmin[0] = b.min.x; nd.bmin[1] = b.min.y; nd.bmin[2] = b.min.z;
        nd.bmax[0] = b.max.x; nd.bmax[1] = b.max.y; nd.bmax[2] = b.max.z;
        nd.offset = start; nd.n_primitives = n;
        nodes.push_back(nd);
        return (uint32_t)nodes.size() - 1;
    }
    uint32_t partition_by_axis(uint32_t start, uint32_t end, int axis, float split_pos) {  // bvh.rs:389-409
        size_t left = start, right = end;
        while (left < right) {
            float c = axis_value(pc[indices[left]], axis);
            if (c < split_pos) left++;
            else { right--; std::swap(indices[left], indices[right]); }
        }
        return (uint32_t)left;
    }
    uint32_t push_split(const Bounds3& b, int axis, uint32_t start, uint32_t mid, uint32_t end) {  // bvh.rs:360-387
        BvhNode nd; std::memset(&nd, 0, sizeof nd);
        nd.bmin[0] = b.min.x; nd.bmin[1] = b.min.y; nd.bmin[2] = b.min.z;
        nd.bmax[0] = b.max.x; nd.bmax[1] = b.max.y; nd.bmax[2] = b.max.z;
        nd.axis = (uint8_t)axis;
        nodes.push_back(nd);
        uint32_t node_idx = (uint32_t)nodes.size() - 1;
        build(start, mid);
        uint32_t right_idx = (uint32_t)nodes.size();
        build(mid, end);
        nodes[node_idx].offset = right_idx;
        return node_idx;
    }
    uint32_t build(uint32_t start, uint32_t end) {  // bvh.rs:180-346
        size_t n = end - start;
        Bounds3 bounds = Bounds3::empty(), cb = Bounds3::empty();
        for (uint32_t k = start; k < end; ++k) {
            uint32_t i = indices[k];
            bounds = bounds.unite(pb[i]);
            cb = cb.extend(pc[i]);
        }
        if (n == 1) return push_leaf(bounds, start, 1);
        V3 cdiag = cb.diagonal();
        int axis = max_axis(cdiag);
        float extent = axis_value(cdiag, axis);
        if (extent < 1e-9f) return push_leaf(bounds, start, (uint16_t)std::min(n, (size_t)65535));

        struct Bin { uint32_t count; Bounds3 b; } bins[BINS];
        for (int i = 0; i < BINS; ++i) { bins[i].count = 0; bins[i].b = Bounds3::empty(); }
        float centroid_min = axis_value(cb.min, axis);
        float scale = (float)BINS / extent;
        for (uint32_t k = start; k < end; ++k) {
            uint32_t i = indices[k];
            float c = axis_value(pc[i], axis);
            float fb = (c - centroid_min) * scale;
            // Rust `as i32` saturates (NaN -> 0).
            int32_t b;
            if (std::isnan(fb)) b = 0;
            else if (fb >= 2147483647.0f) b = 2147483647;
            else if (fb <= -2147483648.0f) b = (-2147483647 - 1);
            else b = (int32_t)fb;
            if (b < 0) b = 0;
            if (b >= BINS) b = BINS - 1;
            bins[b].count += 1;
            bins[b].b = bins[b].b.unite(pb[i]);
        }
        uint32_t left_count[BINS - 1], right_count[BINS - 1];
        Bounds3 left_bounds[BINS - 1], right_bounds[BINS - 1];
        uint32_t acc = 0; Bounds3 accb = Bounds3::empty();
        for (int i = 0; i < BINS - 1; ++i) {
            acc += bins[i].count; accb = accb.unite(bins[i].b);
            left_count[i] = acc; left_bounds[i] = accb;
        }
        acc = 0; accb = Bounds3::empty();
        for (int i = BINS - 2; i >= 0; --i) {
            acc += bins[i + 1].count; accb = accb.unite(bins[i + 1].b);
            right_count[i] = acc; right_bounds[i] = accb;
        }
        float parent_area = fmax_(bounds.surface_area(), 1e-9f);
        float best_cost = INF; int best_split = 0;
        for (int i = 0; i < BINS - 1; ++i) {
            if (left_count[i] == 0 || right_count[i] == 0) continue;
            float cost = TRAVERSAL_COST + INTERSECT_COST *
                ((float)left_count[i] * left_bounds[i].surface_area() +
                 (float)right_count[i] * right_bounds[i].surface_area()) / parent_area;
            if (cost < best_cost) { best_cost = cost; best_split = i; }
        }
        float leaf_cost = INTERSECT_COST * (float)n;
        if (!std::isfinite(best_cost)) {
            float mid_pos = centroid_min + 0.5f * extent;
            uint32_t mid = partition_by_axis(start, end, axis, mid_pos);
            if (mid != start && mid != end) return push_split(bounds, axis, start, mid, end);
            if (n <= MAX_PRIMS_PER_LEAF) return push_leaf(bounds, start, (uint16_t)n);
            mid = start + (uint32_t)n / 2;
            return push_split(bounds, axis, start, mid, end);
        }
        if (n <= MAX_PRIMS_PER_LEAF && best_cost >= leaf_cost) return push_leaf(bounds, start, (uint16_t)n);
        float split_pos = centroid_min + (float)(best_split + 1) * extent / (float)BINS;
        uint32_t mid = partition_by_axis(start, end, axis, split_pos);
        if (mid == start || mid == end) {
            if (n <= MAX_PRIMS_PER_LEAF) return push_leaf(bounds, start, (uint16_t)n);
            mid = start + (uint32_t)n / 2;
            return push_split(bounds, axis, start, mid, end);
        }
        return push_split(bounds, axis, start, mid, end);
    }
};

// ---------------------------------------------------------------------------
// Meshes — crates/pyre/src/geometry/mesh.rs:5-178
// ---------------------------------------------------------------------------
struct Hit {  // SurfaceInteraction (geometry/mod.rs:12-17) + reported ids
    float t = 0.0f;
    V3 position, normal;
    uint32_t tri = 0;
    float u = 0.0f, v = 0.0f;
};

// mesh.rs:153-178
static inline bool moller_trumbore(const Ray& ray, V3 v0, V3 v1, V3 v2, float* t_out, float* u_out, float* v_out) {
    V3 edge1 = v1 - v0, edge2 = v2 - v0;
    V3 h = cross(ray.direction, edge2);
    float a = dot(edge1, h);
    if (std::fabs(a) < 1e-8f) return false;
    float f = 1.0f / a;
    V3 s = ray.origin - v0;
    float u = f * dot(s, h);
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    V3 q = cross(s, edge1);
    float v = f * dot(ray.direction, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    float t = f * dot(edge2, q);
    if (t > ray.t_min && t < ray.t_max) { *t_out = t; *u_out = u; *v_out = v; return true; }
    return false;
}

// bvh.rs:146-153
static inline bool ray_aabb(const Ray& ray, const BvhNode& b, V3 inv_dir, float t_max) {
    V3 bmin(b.bmin[0], b.bmin[1], b.bmin[2]), bmax(b.bmax[0], b.bmax[1], b.bmax[2]);
    V3 t1 = (bmin - ray.origin) * inv_dir;
    V3 t2 = (bmax - ray.origin) * inv_dir;
    float tmin = fmax_(max_element(vmin(t1, t2)), ray.t_min);
    float tmax = fmin_(min_element(vmax(t1, t2)), t_max);
    return tmin <= tmax;
}

struct Mesh {
    std::vector<V3> positions;
    std::vector<uint32_t> indices;
    std::vector<V3> normals;
    bool has_normals = false;
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> prim;
    bool has_motion = false;
    V3 off0, off1;
    uint32_t material_id = 0;

    void build_bvh() {  // MeshInstance::build, mesh.rs:77-87
        size_t n = indices.size() / 3;
        std::vector<Bounds3> bounds(n);
        std::vector<V3> cents(n);
        for (size_t t = 0; t < n; ++t) {
            V3 a = positions[indices[3 * t]], b = positions[indices[3 * t + 1]], c = positions[indices[3 * t + 2]];
            bounds[t] = Bounds3::point(a).extend(b).extend(c);
            cents[t] = (a + b + c) / 3.0f;
        }
        prim.resize(n);
        for (size_t i = 0; i < n; ++i) prim[i] = (uint32_t)i;
        nodes.clear();
        nodes.reserve(2 * std::max(n, (size_t)1));
        if (n > 0) { BvhBuilder b{nodes, prim.data(), bounds.data(), cents.data()}; b.build(0, (uint32_t)n); }
    }
    V3 motion_at(float time) const {  // mesh.rs:53-55
        if (!has_motion) return V3();
        return lerp(off0, off1, clampf(time, 0.0f, 1.0f));
    }

    // MeshInstance::intersect (mesh.rs:110-148) with Bvh::intersect (bvh.rs:86-143).
    // canonical = 0: the reference's visit-order tie rule (first found wins);
    // canonical = 1: ties at equal t resolved to the lowest triangle id.
    bool intersect(const Ray& ray, Hit* out, int canonical, bool any_hit = false) const {
        if (nodes.empty()) return false;
        V3 offset = motion_at(ray.time);
        Ray local = ray;
        if (offset != V3()) local.origin = ray.origin - offset;
        V3 inv_dir = V3(1.0f, 1.0f, 1.0f) / local.direction;
        bool dir_neg[3] = {inv_dir.x < 0.0f, inv_dir.y < 0.0f, inv_dir.z < 0.0f};
        bool found = false;
        float t_max = local.t_max;
        uint32_t stack[64]; stack[0] = 0; size_t sp = 1;
        while (sp > 0) {
            sp--;
            uint32_t idx = stack[sp];
            const BvhNode& node = nodes[idx];
            if (!ray_aabb(local, node, inv_dir, t_max)) continue;
            if (node.n_primitives > 0) {
                for (uint32_t k = node.offset; k < node.offset + node.n_primitives; ++k) {
                    uint32_t tri = prim[k];
                    Ray tight = local;
                    // Reference: the bound is exclusive (bvh.rs:116-119). Canonical
                    // mode also admits t equal to the best hit found in this
                    // instance so that the lower triangle id can win the tie.
                    tight.t_max = (canonical && found) ? std::nextafter(t_max, INF) : t_max;
                    V3 v0 = positions[indices[3 * tri]], v1 = positions[indices[3 * tri + 1]], v2 = positions[indices[3 * tri + 2]];
                    float t, u, v;
                    if (!moller_trumbore(tight, v0, v1, v2, &t, &u, &v)) continue;
                    if (!(t >= local.t_min)) continue;
                    bool better = t < t_max || (canonical && found && t == t_max && tri < out->tri);
                    if (!better) continue;
                    t_max = t; found = true;
                    out->t = t; out->tri = tri; out->u = u; out->v = v;
                    if (any_hit) return true;
                }
            } else {
                uint32_t left = idx + 1, right = node.offset;
                if (dir_neg[node.axis]) { stack[sp++] = left; stack[sp++] = right; }
                else { stack[sp++] = right; stack[sp++] = left; }
            }
        }
        if (!found) return false;
        // Position and normal from the chosen triangle (mesh.rs:126-136).
        uint32_t tri = out->tri;
        uint32_t a = indices[3 * tri], b = indices[3 * tri + 1], c = indices[3 * tri + 2];
        out->position = local.at(out->t);
        if (has_normals) {
            float w = 1.0f - out->u - out->v;
            out->normal = normalize(w * normals[a] + out->u * normals[b] + out->v * normals[c]);
        } else {
            out->normal = normalize(cross(positions[b] - positions[a], positions[c] - positions[a]));
        }
        if (offset != V3()) out->position = out->position + offset;
        return true;
    }
};

// ---------------------------------------------------------------------------
// Materials — crates/pyre/src/material.rs:42-317
// ---------------------------------------------------------------------------
static inline float luminance(V3 c) { return dot(c, V3(0.2126f, 0.7152f, 0.0722f)); }
static inline V3 cosine_sample_hemisphere(V2 u) {  // material.rs:239-246
    float r = std::sqrt(u.x);
    float phi = 2.0f * PI * u.y;
    return V3(r * std::cos(phi), r * std::sin(phi), std::sqrt(fmax_(1.0f - u.x, 0.0f)));
}
static inline float ggx_d(V3 h, float alpha) {  // material.rs:249-256
    if (h.z <= 0.0f) return 0.0f;
    float a2 = alpha * alpha;
    float denom = h.z * h.z * (a2 - 1.0f) + 1.0f;
    return a2 / (PI * denom * denom);
}
static inline V3 schlick_fresnel(float cos_d, V3 f0) {  // material.rs:259-262
    float c = clampf(cos_d, 0.0f, 1.0f);
    return f0 + (V3(1, 1, 1) - f0) * powi5(1.0f - c);
}
static inline float ggx_lambda(V3 v, float alpha) {  // material.rs:264-272
    float cos2 = v.z * v.z;
    if (cos2 >= 1.0f) return 0.0f;
    float a2 = alpha * alpha;
    float tan2 = (1.0f - cos2) / fmax_(cos2, 1e-8f);
    return 0.5f * (-1.0f + std::sqrt(1.0f + a2 * tan2));
}
static inline float ggx_g1(V3 v, float alpha) { return 1.0f / (1.0f + ggx_lambda(v, alpha)); }
static inline float ggx_g2(V3 wo, V3 wi, float alpha) { return 1.0f / (1.0f + ggx_lambda(wo, alpha) + ggx_lambda(wi, alpha)); }
static inline V3 reflect(V3 v, V3 n) { return 2.0f * dot(v, n) * n - v; }
static V3 sample_ggx_vndf(V3 wo, float alpha, V2 u) {  // material.rs:291-317
    V3 vh = normalize(V3(alpha * wo.x, alpha * wo.y, wo.z));
    float lensq = vh.x * vh.x + vh.y * vh.y;
    V3 t1 = lensq > 0.0f ? V3(-vh.y, vh.x, 0.0f) / std::sqrt(lensq) : V3(1, 0, 0);
    V3 t2 = cross(vh, t1);
    float r = std::sqrt(u.x);
    float phi = 2.0f * PI * u.y;
    float t1c = r * std::cos(phi);
    float t2c = r * std::sin(phi);
    float s = 0.5f * (1.0f + vh.z);
    t2c = (1.0f - s) * std::sqrt(fmax_(1.0f - t1c * t1c, 0.0f)) + s * t2c;
    V3 nh = t1c * t1 + t2c * t2 + std::sqrt(fmax_(1.0f - t1c * t1c - t2c * t2c, 0.0f)) * vh;
    return normalize(V3(alpha * nh.x, alpha * nh.y, fmax_(nh.z, 0.0f)));
}

enum { MAT_LAMBERTIAN = 0, MAT_DISNEY = 1 };
struct Material {
    int kind = MAT_LAMBERTIAN;
    V3 albedo;  // Lambertian albedo or Disney base_color
    float metallic = 0, roughness = 0, specular = 0;

    V3 albedo_aov() const { return albedo; }
    float alpha() const { return fmax_(roughness * roughness, 1e-3f); }
    V3 f0() const { return lerp(V3::splat(0.08f * specular), albedo, metallic); }
    void lobe_weights(float* pd, float* ps) const {  // material.rs:112-121
        float diff = (1.0f - metallic) * luminance(albedo);
        float spec = fmax_(luminance(f0()), 0.04f);
        float total = diff + spec;
        if (total > 0.0f) { *pd = diff / total; *ps = spec / total; }
        else { *pd = 1.0f; *ps = 0.0f; }
    }
    V3 eval_diffuse(V3 wo, V3 wi) const {  // material.rs:125-138
        if (wo.z <= 0.0f || wi.z <= 0.0f || metallic >= 1.0f) return V3();
        V3 h = normalize_or_zero(wo + wi);
        if (length_squared(h) < 1e-10f) return V3();
        float cos_d = clampf(dot(wi, h), 0.0f, 1.0f);
        float fd90 = 0.5f + 2.0f * roughness * cos_d * cos_d;
        float fd_v = 1.0f + (fd90 - 1.0f) * powi5(fmax_(1.0f - wo.z, 0.0f));
        float fd_l = 1.0f + (fd90 - 1.0f) * powi5(fmax_(1.0f - wi.z, 0.0f));
        return albedo * (1.0f - metallic) / PI * fd_v * fd_l;
    }
    V3 eval_specular(V3 wo, V3 wi) const {  // material.rs:142-155
        if (wo.z <= 0.0f || wi.z <= 0.0f) return V3();
        V3 h = normalize_or_zero(wo + wi);
        if (length_squared(h) < 1e-10f || h.z <= 0.0f) return V3();
        float a = alpha();
        float d = ggx_d(h, a);
        V3 f = schlick_fresnel(fmax_(dot(wi, h), 0.0f), f0());
        float g = ggx_g2(wo, wi, a);
        return d * f * g / (4.0f * wo.z * wi.z);
    }
    float pdf_diffuse(V3, V3 wi) const { return wi.z <= 0.0f ? 0.0f : wi.z / PI; }
    float pdf_specular(V3 wo, V3 wi) const {  // material.rs:168-180
        if (wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
        V3 h = normalize_or_zero(wo + wi);
        if (length_squared(h) < 1e-10f || h.z <= 0.0f) return 0.0f;
        float a = alpha();
        float d = ggx_d(h, a);
        float g1 = ggx_g1(wo, a);
        return g1 * d / (4.0f * wo.z);
    }
    V3 eval(V3 wo, V3 wi) const {
        if (kind == MAT_LAMBERTIAN) {  // material.rs:52-58
            if (wo.z <= 0.0f || wi.z <= 0.0f) return V3();
            return albedo / PI;
        }
        return eval_diffuse(wo, wi) + eval_specular(wo, wi);
    }
    float pdf(V3 wo, V3 wi) const {
        if (kind == MAT_LAMBERTIAN) {  // material.rs:60-66
            if (wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
            return wi.z / PI;
        }
        float pd, ps; lobe_weights(&pd, &ps);
        return pd * pdf_diffuse(wo, wi) + ps * pdf_specular(wo, wi);
    }
    bool sample(V3 wo, V2 u, V3* wi_out, V3* f_out, float* pdf_out) const {
        if (kind == MAT_LAMBERTIAN) {  // material.rs:68-76
            if (wo.z <= 0.0f) return false;
            V3 wi = cosine_sample_hemisphere(u);
            *wi_out = wi; *pdf_out = wi.z / PI; *f_out = albedo / PI;
            return true;
        }
        // material.rs:197-225
        if (wo.z <= 0.0f) return false;
        float pd, ps; lobe_weights(&pd, &ps);
        if (pd + ps <= 0.0f) return false;
        V3 wi;
        if (u.x < pd) {
            V2 ur; ur.x = fmin_(u.x / pd, 1.0f - 1e-7f); ur.y = u.y;
            wi = cosine_sample_hemisphere(ur);
        } else {
            V2 ur; ur.x = fmin_((u.x - pd) / ps, 1.0f - 1e-7f); ur.y = u.y;
            V3 h = sample_ggx_vndf(wo, alpha(), ur);
            wi = reflect(wo, h);
        }
        if (wi.z <= 0.0f) return false;
        float p = pdf(wo, wi);
        if (p <= 0.0f) return false;
        *wi_out = wi; *f_out = eval(wo, wi); *pdf_out = p;
        return true;
    }
};

// ---------------------------------------------------------------------------
// Lights — crates/pyre/src/light.rs:46-350
// ---------------------------------------------------------------------------
struct QuadLight {  // DiffuseAreaQuadLight, light.rs:46-162
    V3 p0, edge_u, edge_v, crs, normal, emission;
    float inv_cross_len_sq = 0, area = 0;
    static QuadLight make(V3 p0, V3 eu, V3 ev, V3 em) {
        QuadLight q; q.p0 = p0; q.edge_u = eu; q.edge_v = ev; q.emission = em;
        q.crs = cross(eu, ev);
        q.area = length(q.crs);
        q.inv_cross_len_sq = 1.0f / length_squared(q.crs);
        q.normal = normalize(q.crs);
        return q;
    }
    bool intersect_plane(V3 origin, V3 dir, float t_min, float t_max, float* t_out, V3* p_out) const {
        float denom = dot(dir, normal);
        if (std::fabs(denom) < 1e-9f) return false;
        float t = dot(p0 - origin, normal) / denom;
        if (t < t_min || t > t_max) return false;
        V3 p = origin + t * dir;
        V3 d = p - p0;
        float alpha = dot(cross(d, edge_v), crs) * inv_cross_len_sq;
        if (!(alpha >= 0.0f && alpha <= 1.0f)) return false;
        float beta = dot(cross(edge_u, d), crs) * inv_cross_len_sq;
        if (!(beta >= 0.0f && beta <= 1.0f)) return false;
        *t_out = t; *p_out = p;
        return true;
    }
    bool sample(V3 from, V2 u, V3* pos, V3* wi_out, float* pdf_out, V3* li) const {  // light.rs:111-133
        V3 p = p0 + u.x * edge_u + u.y * edge_v;
        V3 to_light = p - from;
        float dist2 = length_squared(to_light);
        if (dist2 <= 0.0f) return false;
        float dist = std::sqrt(dist2);
        V3 wi = to_light / dist;
        float cos_light = -dot(wi, normal);
        if (cos_light <= 0.0f) return false;
        *pdf_out = dist2 / (cos_light * area);
        *pos = p; *wi_out = wi; *li = emission;
        return true;
    }
    float pdf(V3 from, V3 wi) const {  // light.rs:135-144
        float t; V3 p;
        if (!intersect_plane(from, wi, 1e-4f, INF, &t, &p)) return 0.0f;
        float cos_light = -dot(wi, normal);
        if (cos_light <= 0.0f) return 0.0f;
        return t * t / (cos_light * area);
    }
    V3 le(V3 n, V3 wo) const { return dot(n, wo) > 0.0f ? emission : V3(); }  // light.rs:146-152
};

struct Env {  // HdriEnvironmentLight, light.rs:205-350
    uint32_t width = 0, height = 0;
    std::vector<V3> pixels;
    Distribution2D dist;
    float intensity = 1.0f;
    void init(uint32_t w, uint32_t h, const float* rgb, float inten) {  // light.rs:214-242
        width = w; height = h; intensity = inten;
        pixels.resize((size_t)w * h);
        for (size_t i = 0; i < pixels.size(); ++i) pixels[i] = V3(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
        std::vector<float> weights;
        weights.reserve((size_t)w * h);
        for (uint32_t y = 0; y < h; ++y) {
            float theta = ((float)y + 0.5f) / (float)h * PI;
            float sin_theta = fmax_(std::sin(theta), 0.0f);
            for (uint32_t x = 0; x < w; ++x) {
                V3 p = pixels[(size_t)y * w + x];
                float lum = 0.21267f * p.x + 0.71516f * p.y + 0.07217f * p.z;
                weights.push_back(fmax_(lum, 0.0f) * sin_theta);
            }
        }
        dist = Distribution2D(weights.data(), w, h);
    }
    static V2 dir_to_uv(V3 wi) {  // light.rs:274-280
        float theta = std::acos(clampf(wi.y, -1.0f, 1.0f));
        float phi = std::atan2(wi.z, wi.x);
        V2 uv; uv.x = (phi + PI) * FRAC_1_PI * 0.5f; uv.y = theta * FRAC_1_PI; return uv;
    }
    static V3 uv_to_dir(V2 uv) {  // light.rs:282-287
        float phi = uv.x * TAU - PI;
        float theta = uv.y * PI;
        float st = std::sin(theta);
        return V3(st * std::cos(phi), std::cos(theta), st * std::sin(phi));
    }
    static float fract(float x) { return x - std::trunc(x); }
    static int32_t as_i32(float f) {
        if (std::isnan(f)) return 0;
        if (f >= 2147483647.0f) return 2147483647;
        if (f <= -2147483648.0f) return -2147483647 - 1;
        return (int32_t)f;
    }
    static int32_t rem_euclid(int32_t a, int32_t b) { int32_t r = a % b; return r < 0 ? r + b : r; }
    V3 sample_texture(V2 uv) const {  // light.rs:290-314
        int32_t w = (int32_t)width, h = (int32_t)height;
        float u = fract(fract(uv.x) + 1.0f);
        float v = clampf(uv.y, 0.0f, 1.0f);
        float fx = u * (float)w - 0.5f;
        float fy = clampf(v * (float)h - 0.5f, 0.0f, (float)h - 1.0f);
        int32_t x0i = as_i32(std::floor(fx));
        int32_t y0i = as_i32(std::floor(fy));
        float dx = fx - (float)x0i;
        float dy = fy - (float)y0i;
        int32_t x0 = rem_euclid(x0i, w);
        int32_t x1 = rem_euclid(x0 + 1, w);
        int32_t y0 = std::min(std::max(y0i, 0), h - 1);
        int32_t y1 = std::min(y0 + 1, h - 1);
        auto px = [&](int32_t x, int32_t y) { return pixels[(size_t)y * width + (size_t)x]; };
        return px(x0, y0) * ((1.0f - dx) * (1.0f - dy)) + px(x1, y0) * (dx * (1.0f - dy)) +
               px(x0, y1) * ((1.0f - dx) * dy) + px(x1, y1) * (dx * dy);
    }
    V3 le(V3 wi) const { return sample_texture(dir_to_uv(wi)) * intensity; }  // light.rs:318-320
    void sample(V2 u, V3* wi, V3* li, float* pdf) const {  // light.rs:322-338
        float pdf_uv;
        V2 uv = dist.sample_continuous(u, &pdf_uv);
        *wi = uv_to_dir(uv);
        float theta = uv.y * PI;
        float st = std::sin(theta);
        *pdf = (st > 1e-6f && pdf_uv > 0.0f) ? pdf_uv / (2.0f * PI * PI * st) : 0.0f;
        *li = sample_texture(uv) * intensity;
    }
    float pdf(V3 wi) const {  // light.rs:340-349
        V2 uv = dir_to_uv(wi);
        float theta = uv.y * PI;
        float st = std::sin(theta);
        if (st < 1e-6f) return 0.0f;
        return dist.pdf_at(uv) / (2.0f * PI * PI * st);
    }
};

// ---------------------------------------------------------------------------
// Scene — crates/pyre/src/scene.rs:19-152
// ---------------------------------------------------------------------------
struct SceneHit {
    Hit hit; int is_light = 0; uint32_t id = 0; uint32_t material_id = 0;
};

struct Scene {
    std::vector<Mesh> prims;
    std::vector<Material> materials;
    std::vector<QuadLight> lights;
    bool has_env = false;
    Env env;

    // scene.rs:57-97
    bool intersect(const Ray& ray, SceneHit* out, int canonical) const {
        bool found = false;
        float t_max = ray.t_max;
        for (size_t id = 0; id < prims.size(); ++id) {
            Ray r = ray; r.t_max = t_max;
            Hit h;
            // Strict `<` keeps the earlier instance on an exact tie, which is
            // already the canonical (lowest instance id) choice.
            bool ok = prims[id].intersect(r, &h, canonical);
            if (ok && h.t < t_max) {
                t_max = h.t; found = true;
                out->hit = h; out->is_light = 0; out->id = (uint32_t)id; out->material_id = prims[id].material_id;
            }
        }
        for (size_t id = 0; id < lights.size(); ++id) {
            float t; V3 p;
            if (lights[id].intersect_plane(ray.origin, ray.direction, ray.t_min, t_max, &t, &p) && t < t_max) {
                t_max = t; found = true;
                out->hit.t = t; out->hit.position = p; out->hit.normal = lights[id].normal;
                out->hit.tri = 0; out->hit.u = 0; out->hit.v = 0;
                out->is_light = 1; out->id = (uint32_t)id; out->material_id = 0;
            }
        }
        return found;
    }
    bool any_prim_hit(const Ray& ray) const {
        Hit h;
        for (const Mesh& m : prims) if (m.intersect(ray, &h, 0, true)) return true;
        return false;
    }
    bool occluded_dir(V3 from, V3 dir, float time) const {  // scene.rs:102-116
        Ray r; r.origin = from; r.direction = dir; r.t_min = 1e-3f; r.t_max = INF; r.time = time;
        return any_prim_hit(r);
    }
    bool occluded(V3 from, V3 to, float time) const {  // scene.rs:120-140
        V3 tf = to - from;
        float dist = length(tf);
        if (dist <= 0.0f) return false;
        V3 dir = tf / dist;
        Ray r; r.origin = from; r.direction = dir; r.t_min = 1e-3f; r.t_max = dist - 1e-3f; r.time = time;
        return any_prim_hit(r);
    }
};

// ---------------------------------------------------------------------------
// Integrator — crates/pyre/src/integrator.rs:14-240
// ---------------------------------------------------------------------------
struct PixelSample { V3 radiance, albedo, normal; float depth; };
static const float RAY_EPS = 1e-3f;

static inline float power_heuristic(float pa, float pb) {  // integrator.rs:234-240
    float a2 = pa * pa, b2 = pb * pb, denom = a2 + b2;
    return denom > 0.0f ? a2 / denom : 0.0f;
}

// integrator.rs:57-232
static PixelSample integrate(Ray ray, const Scene& scene, Sampler& sampler, uint32_t max_depth, uint32_t min_rr_depth,
                             int* bounces_out = nullptr) {
    V3 l, beta(1, 1, 1);
    float last_pdf_bsdf = 0.0f;
    bool last_was_specular = true;
    V3 aov_albedo, aov_normal; float aov_depth = 0.0f; bool aovs_captured = false;
    int bounces = 0;
    for (uint32_t depth = 0; depth < max_depth; ++depth) {
        SceneHit hit;
        bounces++;
        if (!scene.intersect(ray, &hit, 0)) {
            if (scene.has_env) {
                V3 le = scene.env.le(ray.direction);
                if (le != V3()) {
                    if (last_was_specular) l = l + beta * le;
                    else {
                        float pdf_env = scene.env.pdf(ray.direction);
                        float w = power_heuristic(last_pdf_bsdf, pdf_env);
                        l = l + beta * le * w;
                    }
                }
            }
            break;
        }
        if (!aovs_captured) {
            aovs_captured = true;
            aov_normal = hit.hit.normal;
            aov_depth = hit.hit.t;
            aov_albedo = hit.is_light ? V3(1, 1, 1) : scene.materials[hit.material_id].albedo_aov();
        }
        if (hit.is_light) {
            const QuadLight& light = scene.lights[hit.id];
            V3 le = light.le(hit.hit.normal, -ray.direction);
            if (last_was_specular) l = l + beta * le;
            else {
                float pdf_light = light.pdf(ray.origin, ray.direction);
                float w = power_heuristic(last_pdf_bsdf, pdf_light);
                l = l + beta * le * w;
            }
            break;
        }
        const Material& material = scene.materials[hit.material_id];
        V3 p = hit.hit.position, ns = hit.hit.normal;
        Frame frame = Frame::from_normal(ns);
        V3 wo_local = frame.to_local(-ray.direction);
        if (wo_local.z <= 0.0f) break;

        for (const QuadLight& light : scene.lights) {
            V2 u = sampler.next_vec2();
            V3 lpos, lwi, lli; float lpdf;
            if (!light.sample(p, u, &lpos, &lwi, &lpdf, &lli)) continue;
            if (lpdf <= 0.0f || lli == V3()) continue;
            V3 wi_local = frame.to_local(lwi);
            if (wi_local.z <= 0.0f) continue;
            V3 f = material.eval(wo_local, wi_local);
            if (f == V3()) continue;
            V3 p_offset = p + RAY_EPS * ns;
            V3 target = lpos - RAY_EPS * lwi;
            if (scene.occluded(p_offset, target, ray.time)) continue;
            float pdf_bsdf = material.pdf(wo_local, wi_local);
            float w = power_heuristic(lpdf, pdf_bsdf);
            l = l + beta * f * lli * wi_local.z * w / lpdf;
        }
        if (scene.has_env) {
            V2 u = sampler.next_vec2();
            V3 ewi, eli; float epdf;
            scene.env.sample(u, &ewi, &eli, &epdf);
            if (epdf > 0.0f && eli != V3()) {
                V3 wi_local = frame.to_local(ewi);
                if (wi_local.z > 0.0f) {
                    V3 f = material.eval(wo_local, wi_local);
                    if (f != V3()) {
                        V3 p_offset = p + RAY_EPS * ns;
                        if (!scene.occluded_dir(p_offset, ewi, ray.time)) {
                            float pdf_bsdf = material.pdf(wo_local, wi_local);
                            float w = power_heuristic(epdf, pdf_bsdf);
                            l = l + beta * f * eli * wi_local.z * w / epdf;
                        }
                    }
                }
            }
        }
        V3 bwi, bf; float bpdf;
        if (!material.sample(wo_local, sampler.next_vec2(), &bwi, &bf, &bpdf)) break;
        if (bpdf <= 0.0f) break;
        float cos_wi = std::fabs(bwi.z);
        if (cos_wi == 0.0f) break;
        beta = beta * (bf * cos_wi / bpdf);
        if (depth >= min_rr_depth) {
            float q = clampf(1.0f - max_element(beta), 0.05f, 0.95f);
            if (sampler.next_f32() < q) break;
            beta = beta / (1.0f - q);
        }
        last_pdf_bsdf = bpdf;
        last_was_specular = false;
        V3 wi_world = frame.to_world(bwi);
        Ray nr; nr.origin = p + RAY_EPS * ns; nr.direction = wi_world; nr.t_min = 1e-4f; nr.t_max = INF; nr.time = ray.time;
        ray = nr;
    }
    if (bounces_out) *bounces_out = bounces;
    PixelSample ps; ps.radiance = l; ps.albedo = aov_albedo; ps.normal = aov_normal; ps.depth = aov_depth;
    return ps;
}

// One sample of the CLI render loop (crates/pyre-cli/src/main.rs:261-274).
static PixelSample render_sample(const Scene& scene, const Camera& cam, uint32_t width, uint32_t height,
                                 uint32_t x, uint32_t y, uint32_t s, uint32_t max_depth, uint32_t min_rr, int* bounces) {
    Sampler sampler(pixel_seed(x, y, s));
    float jx = sampler.next_f32();
    float jy = sampler.next_f32();
    V2 ndc;
    ndc.x = 2.0f * ((float)x + jx) / (float)width - 1.0f;
    ndc.y = 1.0f - 2.0f * ((float)y + jy) / (float)height;
    V2 lens = sampler.next_vec2();
    float time = sampler.next_f32();
    Ray ray = cam.generate_ray(ndc, lens, time);
    return integrate(ray, scene, sampler, max_depth, min_rr, bounces);
}

// ---------------------------------------------------------------------------
// Forward-mode gradient of the integrator (no reference counterpart).
//
// Same path as integrate() (same sampler draws and decisions), with the
// detached-sampling convention: the BSDF values f (throughput and NEE) and
// the emitted environment radiance carry derivatives; pdfs, MIS weights,
// lobe choice, Russian roulette and the environment's sampling tables are
// constants. Tangents are all material parameters (6 per material: base
// r,g,b, metallic, roughness, specular) followed by all environment texels
// (3 per texel). The throughput carries a dense tangent vector per channel.
// ---------------------------------------------------------------------------
struct Dual6 {
    float v; float d[6];
    Dual6() : v(0) { for (float& x : d) x = 0; }
    Dual6(float a) : v(a) { for (float& x : d) x = 0; }
    static Dual6 var(float a, int k) { Dual6 r(a); r.d[k] = 1.0f; return r; }
};
static inline Dual6 operator+(Dual6 a, Dual6 b) { Dual6 r(a.v + b.v); for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] + b.d[k]; return r; }
static inline Dual6 operator-(Dual6 a, Dual6 b) { Dual6 r(a.v - b.v); for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] - b.d[k]; return r; }
static inline Dual6 operator*(Dual6 a, Dual6 b) { Dual6 r(a.v * b.v); for (int k = 0; k < 6; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r; }
static inline Dual6 operator/(Dual6 a, Dual6 b) {
    Dual6 r(a.v / b.v);
    for (int k = 0; k < 6; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
    return r;
}
static inline Dual6 dsqrt(Dual6 a) {
    Dual6 r(std::sqrt(a.v));
    for (int k = 0; k < 6; ++k) r.d[k] = r.v > 0 ? a.d[k] / (2.0f * r.v) : 0.0f;
    return r;
}

// f(wo, wi) and J[c][k] = d f_c / d param_k (material.rs:52-58, 125-155).
static void eval_jacobian(const Material& m, V3 wo, V3 wi, float J[3][6]) {
    for (int c = 0; c < 3; ++c) for (int k = 0; k < 6; ++k) J[c][k] = 0.0f;
    if (m.kind == MAT_LAMBERTIAN) {
        if (wo.z <= 0.0f || wi.z <= 0.0f) return;
        J[0][0] = J[1][1] = J[2][2] = 1.0f / PI;
        return;
    }
    Dual6 base[3] = {Dual6::var(m.albedo.x, 0), Dual6::var(m.albedo.y, 1), Dual6::var(m.albedo.z, 2)};
    Dual6 metal = Dual6::var(m.metallic, 3), rough = Dual6::var(m.roughness, 4), spec = Dual6::var(m.specular, 5);
    Dual6 f[3];
    if (!(wo.z <= 0.0f || wi.z <= 0.0f || m.metallic >= 1.0f)) {
        V3 h = normalize_or_zero(wo + wi);
        if (!(length_squared(h) < 1e-10f)) {
            float cos_d = clampf(dot(wi, h), 0.0f, 1.0f);
            Dual6 fd90 = Dual6(0.5f) + Dual6(2.0f) * rough * Dual6(cos_d) * Dual6(cos_d);
            Dual6 fd_v = Dual6(1.0f) + (fd90 - Dual6(1.0f)) * Dual6(powi5(fmax_(1.0f - wo.z, 0.0f)));
            Dual6 fd_l = Dual6(1.0f) + (fd90 - Dual6(1.0f)) * Dual6(powi5(fmax_(1.0f - wi.z, 0.0f)));
            for (int c = 0; c < 3; ++c) f[c] = base[c] * (Dual6(1.0f) - metal) / Dual6(PI) * fd_v * fd_l;
        }
    }
    if (!(wo.z <= 0.0f || wi.z <= 0.0f)) {
        V3 h = normalize_or_zero(wo + wi);
        if (!(length_squared(h) < 1e-10f || h.z <= 0.0f)) {
            Dual6 r2 = rough * rough;
            Dual6 alpha = r2.v >= 1e-3f ? r2 : Dual6(1e-3f);
            Dual6 a2 = alpha * alpha;
            Dual6 denom = Dual6(h.z * h.z) * (a2 - Dual6(1.0f)) + Dual6(1.0f);
            Dual6 D = a2 / (Dual6(PI) * denom * denom);
            auto lambda = [&](V3 v) {
                float cos2 = v.z * v.z;
                if (cos2 >= 1.0f) return Dual6(0.0f);
                float tan2 = (1.0f - cos2) / fmax_(cos2, 1e-8f);
                return Dual6(0.5f) * (Dual6(-1.0f) + dsqrt(Dual6(1.0f) + a2 * Dual6(tan2)));
            };
            Dual6 G = Dual6(1.0f) / (Dual6(1.0f) + lambda(wo) + lambda(wi));
            float c5 = powi5(1.0f - clampf(fmax_(dot(wi, h), 0.0f), 0.0f, 1.0f));
            Dual6 diel = Dual6(0.08f) * spec;
            for (int c = 0; c < 3; ++c) {
                Dual6 f0 = diel * (Dual6(1.0f) - metal) + base[c] * metal;
                Dual6 F = f0 + (Dual6(1.0f) - f0) * Dual6(c5);
                f[c] = f[c] + D * F * G / Dual6(4.0f * wo.z * wi.z);
            }
        }
    }
    for (int c = 0; c < 3; ++c) for (int k = 0; k < 6; ++k) J[c][k] = f[c].d[k];
}

// Bilinear texel weights of Env::sample_texture (light.rs:290-314).
static void texel_weights(const Env& e, V2 uv, uint32_t idx[4], float wt[4]) {
    int32_t w = (int32_t)e.width, h = (int32_t)e.height;
    float u = Env::fract(Env::fract(uv.x) + 1.0f);
    float v = clampf(uv.y, 0.0f, 1.0f);
    float fx = u * (float)w - 0.5f;
    float fy = clampf(v * (float)h - 0.5f, 0.0f, (float)h - 1.0f);
    int32_t x0i = Env::as_i32(std::floor(fx)), y0i = Env::as_i32(std::floor(fy));
    float dx = fx - (float)x0i, dy = fy - (float)y0i;
    int32_t x0 = Env::rem_euclid(x0i, w), x1 = Env::rem_euclid(x0 + 1, w);
    int32_t y0 = std::min(std::max(y0i, 0), h - 1), y1 = std::min(y0 + 1, h - 1);
    idx[0] = (uint32_t)(y0 * w + x0); wt[0] = (1.0f - dx) * (1.0f - dy);
    idx[1] = (uint32_t)(y0 * w + x1); wt[1] = dx * (1.0f - dy);
    idx[2] = (uint32_t)(y1 * w + x0); wt[2] = (1.0f - dx) * dy;
    idx[3] = (uint32_t)(y1 * w + x1); wt[3] = dx * dy;
}

struct GradPath {
    size_t n;                    // tangents carried by the throughput: the material parameters
    std::vector<double> beta_d;  // 3 * n: d beta_c / d theta
    std::vector<double>* grad;   // accumulates delta . dL/dtheta
};

// d(loss) of a term  beta (x) f (x) k  where f carries material m's
// Jacobian J (or none), plus an environment texture factor.
static void add_term(GradPath& G, V3 beta, V3 f, V3 k, V3 delta, int mat, const float (*J)[6],
                     size_t env_base, const Env* env, V2 uv, V3 kenv) {
    const float dv[3] = {delta.x, delta.y, delta.z}, bv[3] = {beta.x, beta.y, beta.z}, fv[3] = {f.x, f.y, f.z},
                kv[3] = {k.x, k.y, k.z};
    std::vector<double>& g = *G.grad;
    for (int c = 0; c < 3; ++c) {
        const double s = (double)dv[c] * fv[c] * kv[c];
        if (s != 0.0) {
            const double* bd = &G.beta_d[(size_t)c * G.n];
            for (size_t t = 0; t < G.n; ++t) g[t] += s * bd[t];
        }
        if (J && mat >= 0) {
            const double w = (double)dv[c] * bv[c] * kv[c];
            for (int p = 0; p < 6; ++p) g[(size_t)mat * 6 + p] += w * J[c][p];
        }
    }
    if (env) {  // term beta * kenv * texture(uv) * intensity
        uint32_t idx[4]; float wt[4];
        texel_weights(*env, uv, idx, wt);
        const float ke[3] = {kenv.x, kenv.y, kenv.z};
        for (int q = 0; q < 4; ++q)
            for (int c = 0; c < 3; ++c)
                g[env_base + 3 * (size_t)idx[q] + c] += (double)dv[c] * bv[c] * ke[c] * wt[q] * env->intensity;
    }
}

static void integrate_grad(Ray ray, const Scene& scene, Sampler& sampler, uint32_t max_depth, uint32_t min_rr,
                           V3 delta, GradPath& G) {
    const size_t env_base = scene.materials.size() * 6;
    V3 beta(1, 1, 1);
    std::fill(G.beta_d.begin(), G.beta_d.end(), 0.0);
    float last_pdf_bsdf = 0.0f;
    bool last_was_specular = true;
    for (uint32_t depth = 0; depth < max_depth; ++depth) {
        SceneHit hit;
        if (!scene.intersect(ray, &hit, 0)) {
            if (scene.has_env) {
                V3 le = scene.env.le(ray.direction);
                if (le != V3()) {
                    float w = last_was_specular ? 1.0f
                                                : power_heuristic(last_pdf_bsdf, scene.env.pdf(ray.direction));
                    // term beta * le * w, le = texture * intensity
                    add_term(G, beta, le, V3(w, w, w), delta, -1, nullptr, env_base, &scene.env,
                             Env::dir_to_uv(ray.direction), V3(w, w, w));
                }
            }
            break;
        }
        if (hit.is_light) {
            const QuadLight& light = scene.lights[hit.id];
            V3 le = light.le(hit.hit.normal, -ray.direction);
            float w = last_was_specular ? 1.0f : power_heuristic(last_pdf_bsdf, light.pdf(ray.origin, ray.direction));
            add_term(G, beta, le, V3(w, w, w), delta, -1, nullptr, 0, nullptr, V2(), V3());
            break;
        }
        const Material& material = scene.materials[hit.material_id];
        const int mat = (int)hit.material_id;
        V3 p = hit.hit.position, ns = hit.hit.normal;
        Frame frame = Frame::from_normal(ns);
        V3 wo_local = frame.to_local(-ray.direction);
        if (wo_local.z <= 0.0f) break;
        for (const QuadLight& light : scene.lights) {
            V2 u = sampler.next_vec2();
            V3 lpos, lwi, lli; float lpdf;
            if (!light.sample(p, u, &lpos, &lwi, &lpdf, &lli)) continue;
            if (lpdf <= 0.0f || lli == V3()) continue;
            V3 wi_local = frame.to_local(lwi);
            if (wi_local.z <= 0.0f) continue;
            V3 f = material.eval(wo_local, wi_local);
            if (f == V3()) continue;
            if (scene.occluded(p + RAY_EPS * ns, lpos - RAY_EPS * lwi, ray.time)) continue;
            float w = power_heuristic(lpdf, material.pdf(wo_local, wi_local));
            float J[3][6];
            eval_jacobian(material, wo_local, wi_local, J);
            add_term(G, beta, f, lli * wi_local.z * w / lpdf, delta, mat, J, 0, nullptr, V2(), V3());
        }
        if (scene.has_env) {
            V2 u = sampler.next_vec2();
            V3 ewi, eli; float epdf;
            scene.env.sample(u, &ewi, &eli, &epdf);
            if (epdf > 0.0f && eli != V3()) {
                V3 wi_local = frame.to_local(ewi);
                if (wi_local.z > 0.0f) {
                    V3 f = material.eval(wo_local, wi_local);
                    if (f != V3() && !scene.occluded_dir(p + RAY_EPS * ns, ewi, ray.time)) {
                        float w = power_heuristic(epdf, material.pdf(wo_local, wi_local));
                        float k = wi_local.z * w / epdf;
                        float J[3][6];
                        eval_jacobian(material, wo_local, wi_local, J);
                        add_term(G, beta, f, eli * k, delta, mat, J, env_base, &scene.env,
                                 Env::dir_to_uv(ewi), f * k);
                    }
                }
            }
        }
        V3 bwi, bf; float bpdf;
        if (!material.sample(wo_local, sampler.next_vec2(), &bwi, &bf, &bpdf)) break;
        if (bpdf <= 0.0f) break;
        float cos_wi = std::fabs(bwi.z);
        if (cos_wi == 0.0f) break;
        float a = cos_wi / bpdf;
        V3 nbeta = beta * (bf * cos_wi / bpdf);
        if (depth >= min_rr) {
            float q = clampf(1.0f - max_element(nbeta), 0.05f, 0.95f);
            if (sampler.next_f32() < q) break;
            nbeta = nbeta / (1.0f - q);
            a = a / (1.0f - q);
        }
        // d beta' = d beta * f * a + beta * a * df
        float J[3][6];
        eval_jacobian(material, wo_local, bwi, J);
        const float fv[3] = {bf.x, bf.y, bf.z}, bv[3] = {beta.x, beta.y, beta.z};
        for (int c = 0; c < 3; ++c) {
            double* bd = &G.beta_d[(size_t)c * G.n];
            const double s = (double)fv[c] * a;
            for (size_t t = 0; t < G.n; ++t) bd[t] *= s;
            for (int q = 0; q < 6; ++q) bd[(size_t)mat * 6 + q] += (double)bv[c] * a * J[c][q];
        }
        beta = nbeta;
        last_pdf_bsdf = bpdf;
        last_was_specular = false;
        Ray nr; nr.origin = p + RAY_EPS * ns; nr.direction = frame.to_world(bwi);
        nr.t_min = 1e-4f; nr.t_max = INF; nr.time = ray.time;
        ray = nr;
    }
}

}  // namespace orc

// ===========================================================================
// C ABI for the Python test harness (ctypes).
// ===========================================================================
using namespace orc;

extern "C" {

uint64_t orc_pixel_seed(uint32_t x, uint32_t y, uint32_t s) { return pixel_seed(x, y, s); }

void orc_rng_stream(uint64_t seed, uint32_t n, float* out_f32, uint64_t* out_state4) {
    Sampler smp(seed);
    if (out_state4) for (int i = 0; i < 4; ++i) out_state4[i] = smp.rng.s[i];
    for (uint32_t i = 0; i < n; ++i) out_f32[i] = smp.next_f32();
}

void orc_rng_u64_stream(uint64_t seed, uint32_t n, uint64_t* out) {
    Xoshiro256pp r = Xoshiro256pp::seed_from_u64(seed);
    for (uint32_t i = 0; i < n; ++i) out[i] = r.next_u64();
}

// Distribution1D: sample at n_u points (t, pdf, bin) for a weight vector.
void orc_dist1d_sample(const float* w, uint32_t n, const float* u, uint32_t n_u,
                       float* t_out, float* pdf_out, uint32_t* bin_out) {
    Distribution1D d(w, n);
    for (uint32_t i = 0; i < n_u; ++i) {
        size_t b; t_out[i] = d.sample_continuous(u[i], &pdf_out[i], &b); bin_out[i] = (uint32_t)b;
    }
}
void orc_dist2d_pdf(const float* w, uint32_t width, uint32_t height, const float* uv, uint32_t n, float* out) {
    Distribution2D d(w, width, height);
    for (uint32_t i = 0; i < n; ++i) { V2 q; q.x = uv[2 * i]; q.y = uv[2 * i + 1]; out[i] = d.pdf_at(q); }
}
void orc_dist2d_sample(const float* w, uint32_t width, uint32_t height, const float* u, uint32_t n, float* uv_out, float* pdf_out) {
    Distribution2D d(w, width, height);
    for (uint32_t i = 0; i < n; ++i) {
        V2 q; q.x = u[2 * i]; q.y = u[2 * i + 1];
        V2 r = d.sample_continuous(q, &pdf_out[i]);
        uv_out[2 * i] = r.x; uv_out[2 * i + 1] = r.y;
    }
}

// BSDF entry points: params = [kind, r, g, b, metallic, roughness, specular]
static Material mat_from(const float* p) {
    Material m; m.kind = (int)p[0]; m.albedo = V3(p[1], p[2], p[3]); m.metallic = p[4]; m.roughness = p[5]; m.specular = p[6];
    return m;
}
void orc_bsdf_eval(const float* params, const float* wo, const float* wi, uint32_t n, float* f_out, float* pdf_out) {
    Material m = mat_from(params);
    for (uint32_t i = 0; i < n; ++i) {
        V3 a(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]), b(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
        V3 f = m.eval(a, b);
        f_out[3 * i] = f.x; f_out[3 * i + 1] = f.y; f_out[3 * i + 2] = f.z;
        pdf_out[i] = m.pdf(a, b);
    }
}
void orc_bsdf_sample(const float* params, const float* wo, const float* u, uint32_t n,
                     uint8_t* ok, float* wi_out, float* f_out, float* pdf_out) {
    Material m = mat_from(params);
    for (uint32_t i = 0; i < n; ++i) {
        V3 a(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
        V2 uu; uu.x = u[2 * i]; uu.y = u[2 * i + 1];
        V3 wi, f; float pdf = 0;
        ok[i] = m.sample(a, uu, &wi, &f, &pdf) ? 1 : 0;
        wi_out[3 * i] = wi.x; wi_out[3 * i + 1] = wi.y; wi_out[3 * i + 2] = wi.z;
        f_out[3 * i] = f.x; f_out[3 * i + 1] = f.y; f_out[3 * i + 2] = f.z;
        pdf_out[i] = pdf;
    }
}

// Reference unit-test replay: material.rs:332-387 with the seeded stream.
// Writes per-case |f_check - f| and |p_check - pdf| maxima; returns #sampled.
int orc_disney_consistency(const float* params3x7, uint64_t seed, uint32_t iters, float* max_df, float* max_dp, float* min_pdf, float* min_wiz) {
    Xoshiro256pp rng = Xoshiro256pp::seed_from_u64(seed);
    int count = 0;
    *max_df = 0; *max_dp = 0; *min_pdf = INF; *min_wiz = INF;
    for (int b = 0; b < 3; ++b) {
        Material m = mat_from(params3x7 + 7 * b);
        for (uint32_t it = 0; it < iters; ++it) {
            float cos_t = rng.next_f32() * 0.99f + 0.01f;
            float phi = rng.next_f32() * TAU;
            float sin_t = std::sqrt(1.0f - cos_t * cos_t);
            V3 wo(sin_t * std::cos(phi), sin_t * std::sin(phi), cos_t);
            V2 u; u.x = rng.next_f32(); u.y = rng.next_f32();
            V3 wi, f; float pdf;
            if (!m.sample(wo, u, &wi, &f, &pdf)) continue;
            V3 fc = m.eval(wo, wi); float pc = m.pdf(wo, wi);
            *max_df = std::max(*max_df, length(fc - f));
            *max_dp = std::max(*max_dp, std::fabs(pc - pdf));
            *min_pdf = std::min(*min_pdf, pdf);
            *min_wiz = std::min(*min_wiz, wi.z);
            count++;
        }
    }
    return count;
}

// The (wo, u) draws of that test in order (3 * iters of each), for running the
// same cases through another implementation of the BSDF.
void orc_disney_draws(uint64_t seed, uint32_t iters, float* wo_out, float* u_out) {
    Xoshiro256pp rng = Xoshiro256pp::seed_from_u64(seed);
    for (uint32_t k = 0; k < 3 * iters; ++k) {
        float cos_t = rng.next_f32() * 0.99f + 0.01f;
        float phi = rng.next_f32() * TAU;
        float sin_t = std::sqrt(1.0f - cos_t * cos_t);
        wo_out[3 * k] = sin_t * std::cos(phi);
        wo_out[3 * k + 1] = sin_t * std::sin(phi);
        wo_out[3 * k + 2] = cos_t;
        u_out[2 * k] = rng.next_f32();
        u_out[2 * k + 1] = rng.next_f32();
    }
}

// ---- BVH build (bvh.rs:45-64): nodes_out must hold 2*ntri nodes -----------
uint32_t orc_bvh_build(const float* pos, const uint32_t* idx, uint32_t ntri, void* nodes_out, uint32_t* prim_out) {
    Mesh m;
    uint32_t nv = 0;
    for (uint32_t i = 0; i < 3 * ntri; ++i) nv = std::max(nv, idx[i] + 1);
    m.positions.resize(nv);
    for (uint32_t i = 0; i < nv; ++i) m.positions[i] = V3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    m.indices.assign(idx, idx + 3 * (size_t)ntri);
    m.build_bvh();
    std::memcpy(nodes_out, m.nodes.data(), m.nodes.size() * sizeof(BvhNode));
    std::memcpy(prim_out, m.prim.data(), m.prim.size() * sizeof(uint32_t));
    return (uint32_t)m.nodes.size();
}

// ---- Scene ----------------------------------------------------------------
void* orc_scene_new(void) { return new Scene(); }
void orc_scene_free(void* s) { delete (Scene*)s; }
int orc_scene_add_lambertian(void* s, const float* albedo) {
    Scene* sc = (Scene*)s; Material m; m.kind = MAT_LAMBERTIAN; m.albedo = V3(albedo[0], albedo[1], albedo[2]);
    sc->materials.push_back(m); return (int)sc->materials.size() - 1;
}
int orc_scene_add_disney(void* s, const float* base, float metallic, float roughness, float specular) {
    Scene* sc = (Scene*)s; Material m; m.kind = MAT_DISNEY; m.albedo = V3(base[0], base[1], base[2]);
    m.metallic = metallic; m.roughness = roughness; m.specular = specular;
    sc->materials.push_back(m); return (int)sc->materials.size() - 1;
}
void orc_scene_set_material(void* s, uint32_t id, const float* params7) {
    Scene* sc = (Scene*)s; sc->materials[id] = mat_from(params7);
}
// motion: NULL or [t0.x,t0.y,t0.z,t1.x,t1.y,t1.z]
int orc_scene_add_mesh(void* s, const float* pos, uint32_t nv, const uint32_t* idx, uint32_t ntri,
                       const float* normals, uint32_t material_id, const float* motion) {
    Scene* sc = (Scene*)s;
    sc->prims.emplace_back();
    Mesh& m = sc->prims.back();
    m.positions.resize(nv);
    for (uint32_t i = 0; i < nv; ++i) m.positions[i] = V3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    m.indices.assign(idx, idx + 3 * (size_t)ntri);
    if (normals) {
        m.has_normals = true; m.normals.resize(nv);
        for (uint32_t i = 0; i < nv; ++i) m.normals[i] = V3(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
    }
    m.material_id = material_id;
    if (motion) { m.has_motion = true; m.off0 = V3(motion[0], motion[1], motion[2]); m.off1 = V3(motion[3], motion[4], motion[5]); }
    m.build_bvh();
    return (int)sc->prims.size() - 1;
}
// Builds all meshes' BVHs in parallel instead of one by one (same result).
int orc_scene_add_meshes(void* s, uint32_t n_meshes, const float* const* pos, const uint32_t* nv, const uint32_t* const* idx,
                         const uint32_t* ntri, const float* const* normals, const uint32_t* material_id, const float* const* motion,
                         int nthreads) {
    Scene* sc = (Scene*)s;
    size_t base = sc->prims.size();
    sc->prims.resize(base + n_meshes);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic)
#endif
    for (int k = 0; k < (int)n_meshes; ++k) {
        Mesh& m = sc->prims[base + k];
        m.positions.resize(nv[k]);
        for (uint32_t i = 0; i < nv[k]; ++i) m.positions[i] = V3(pos[k][3 * i], pos[k][3 * i + 1], pos[k][3 * i + 2]);
        m.indices.assign(idx[k], idx[k] + 3 * (size_t)ntri[k]);
        if (normals && normals[k]) {
            m.has_normals = true; m.normals.resize(nv[k]);
            for (uint32_t i = 0; i < nv[k]; ++i) m.normals[i] = V3(normals[k][3 * i], normals[k][3 * i + 1], normals[k][3 * i + 2]);
        }
        m.material_id = material_id[k];
        if (motion && motion[k]) {
            m.has_motion = true;
            m.off0 = V3(motion[k][0], motion[k][1], motion[k][2]);
            m.off1 = V3(motion[k][3], motion[k][4], motion[k][5]);
        }
        m.build_bvh();
    }
    return (int)sc->prims.size();
}
int orc_scene_add_quad_light(void* s, const float* p0, const float* eu, const float* ev, const float* em) {
    Scene* sc = (Scene*)s;
    sc->lights.push_back(QuadLight::make(V3(p0[0], p0[1], p0[2]), V3(eu[0], eu[1], eu[2]), V3(ev[0], ev[1], ev[2]), V3(em[0], em[1], em[2])));
    return (int)sc->lights.size() - 1;
}
void orc_scene_set_env(void* s, uint32_t w, uint32_t h, const float* rgb, float intensity) {
    Scene* sc = (Scene*)s; sc->has_env = true; sc->env.init(w, h, rgb, intensity);
}
void orc_env_query(void* s, const float* u, uint32_t n, float* wi_out, float* li_out, float* pdf_out, float* pdf_back, float* le_back) {
    Scene* sc = (Scene*)s;
    for (uint32_t i = 0; i < n; ++i) {
        V2 uu; uu.x = u[2 * i]; uu.y = u[2 * i + 1];
        V3 wi, li; float pdf;
        sc->env.sample(uu, &wi, &li, &pdf);
        wi_out[3 * i] = wi.x; wi_out[3 * i + 1] = wi.y; wi_out[3 * i + 2] = wi.z;
        li_out[3 * i] = li.x; li_out[3 * i + 1] = li.y; li_out[3 * i + 2] = li.z;
        pdf_out[i] = pdf;
        pdf_back[i] = sc->env.pdf(wi);
        V3 le = sc->env.le(wi);
        le_back[3 * i] = le.x; le_back[3 * i + 1] = le.y; le_back[3 * i + 2] = le.z;
    }
}
uint32_t orc_scene_bvh_nodes(void* s, uint32_t prim, void* nodes_out, uint32_t* prim_out) {
    Scene* sc = (Scene*)s; const Mesh& m = sc->prims[prim];
    if (nodes_out) std::memcpy(nodes_out, m.nodes.data(), m.nodes.size() * sizeof(BvhNode));
    if (prim_out) std::memcpy(prim_out, m.prim.data(), m.prim.size() * sizeof(uint32_t));
    return (uint32_t)m.nodes.size();
}

// ---- Intersection (closest / any) on caller-supplied rays -----------------
// Rays: org[3n], dir[3n] (used as given, not normalized), tmin[n], tmax[n], time[n] (NULL = 0).
// Closest: kind_out 0 = miss, 1 = surface, 2 = light; inst_out = instance or light id.
void orc_intersect(void* s, const float* org, const float* dir, const float* tmin, const float* tmax, const float* time,
                   uint64_t n, int canonical, int nthreads, int32_t* kind_out, int32_t* inst_out, int32_t* tri_out,
                   float* t_out, float* u_out, float* v_out, float* normal_out) {
    Scene* sc = (Scene*)s;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4096)
#endif
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        Ray r; r.origin = V3(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
        r.direction = V3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
        r.t_min = tmin[i]; r.t_max = tmax[i]; r.time = time ? time[i] : 0.0f;
        SceneHit h;
        if (sc->intersect(r, &h, canonical)) {
            kind_out[i] = h.is_light ? 2 : 1; inst_out[i] = (int32_t)h.id;
            tri_out[i] = h.is_light ? -1 : (int32_t)h.hit.tri;
            t_out[i] = h.hit.t; u_out[i] = h.hit.u; v_out[i] = h.hit.v;
            if (normal_out) { normal_out[3 * i] = h.hit.normal.x; normal_out[3 * i + 1] = h.hit.normal.y; normal_out[3 * i + 2] = h.hit.normal.z; }
        } else {
            kind_out[i] = 0; inst_out[i] = -1; tri_out[i] = -1; t_out[i] = INF; u_out[i] = 0; v_out[i] = 0;
        }
    }
}
void orc_occluded(void* s, const float* org, const float* dir, const float* tmin, const float* tmax, const float* time,
                  uint64_t n, int nthreads, uint8_t* out) {
    Scene* sc = (Scene*)s;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4096)
#endif
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        Ray r; r.origin = V3(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
        r.direction = V3(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
        r.t_min = tmin[i]; r.t_max = tmax[i]; r.time = time ? time[i] : 0.0f;
        out[i] = sc->any_prim_hit(r) ? 1 : 0;
    }
}

// ---- Camera ---------------------------------------------------------------
// cam: [thin, ox,oy,oz, tx,ty,tz, ux,uy,uz, vfov_deg, aspect, aperture_radius, focus_distance]
static Camera cam_from(const float* c) {
    return Camera::look_at(V3(c[1], c[2], c[3]), V3(c[4], c[5], c[6]), V3(c[7], c[8], c[9]), c[10], c[11], (int)c[0], c[12], c[13]);
}
void orc_camera_rays(const float* cam, uint32_t width, uint32_t height, const uint32_t* xys, uint32_t n,
                     float* org_out, float* dir_out, float* time_out) {
    Camera c = cam_from(cam);
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t x = xys[3 * i], y = xys[3 * i + 1], s = xys[3 * i + 2];
        Sampler smp(pixel_seed(x, y, s));
        float jx = smp.next_f32(), jy = smp.next_f32();
        V2 ndc; ndc.x = 2.0f * ((float)x + jx) / (float)width - 1.0f; ndc.y = 1.0f - 2.0f * ((float)y + jy) / (float)height;
        V2 lens = smp.next_vec2();
        float time = smp.next_f32();
        Ray r = c.generate_ray(ndc, lens, time);
        org_out[3 * i] = r.origin.x; org_out[3 * i + 1] = r.origin.y; org_out[3 * i + 2] = r.origin.z;
        dir_out[3 * i] = r.direction.x; dir_out[3 * i + 1] = r.direction.y; dir_out[3 * i + 2] = r.direction.z;
        time_out[i] = r.time;
    }
}

// ---- Render (main.rs:253-286 over a crop and a sample range) --------------
// Outputs are crop-sized, row-major: rgb[3*(cy*cw+cx)], albedo[3*..], normal[3*..], depth[..].
// accum64: if non-NULL, receives the FP64 sum of per-sample radiance (not divided).
// Returns total path vertices traced (sum of bounces) for ray counting.
uint64_t orc_render(void* s, const float* cam, uint32_t width, uint32_t height, uint32_t spp_begin, uint32_t spp_end,
                    uint32_t max_depth, uint32_t min_rr_depth, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                    int nthreads, float* rgb, float* albedo, float* normal, float* depth, double* accum64) {
    Scene* sc = (Scene*)s;
    Camera c = cam_from(cam);
    uint32_t cw = x1 - x0, ch = y1 - y0;
    uint32_t spp = spp_end - spp_begin;
    uint64_t total = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : total)
#endif
    for (int64_t pix = 0; pix < (int64_t)cw * ch; ++pix) {
        {
            const int64_t yy = pix / cw;
            const uint32_t xx = (uint32_t)(pix % cw);
            uint32_t x = x0 + xx, y = y0 + (uint32_t)yy;
            float inv_spp = 1.0f / (float)spp;
            V3 rad, alb, nor; float dep = 0.0f;
            double ax = 0, ay = 0, az = 0;
            for (uint32_t sidx = spp_begin; sidx < spp_end; ++sidx) {
                int b = 0;
                PixelSample ps = render_sample(*sc, c, width, height, x, y, sidx, max_depth, min_rr_depth, &b);
                total += (uint64_t)b;
                rad = rad + ps.radiance; alb = alb + ps.albedo; nor = nor + ps.normal; dep += ps.depth;
                ax += ps.radiance.x; ay += ps.radiance.y; az += ps.radiance.z;
            }
            size_t o = (size_t)yy * cw + xx;
            if (rgb) { V3 v = rad * inv_spp; rgb[3 * o] = v.x; rgb[3 * o + 1] = v.y; rgb[3 * o + 2] = v.z; }
            if (albedo) { V3 v = alb * inv_spp; albedo[3 * o] = v.x; albedo[3 * o + 1] = v.y; albedo[3 * o + 2] = v.z; }
            if (normal) { V3 v = nor * inv_spp; normal[3 * o] = v.x; normal[3 * o + 1] = v.y; normal[3 * o + 2] = v.z; }
            if (depth) depth[o] = dep * inv_spp;
            if (accum64) { accum64[3 * o] = ax; accum64[3 * o + 1] = ay; accum64[3 * o + 2] = az; }
        }
    }
    return total;
}

// Forward-mode gradient of the render's loss: dl_di (crop*3) is d loss / d
// film radiance; grad_out (n_mat*6 + env texels*3) receives the gradient.
void orc_render_grad(void* s, const float* cam, uint32_t width, uint32_t height, uint32_t spp_begin,
                     uint32_t spp_end, uint32_t max_depth, uint32_t min_rr_depth, uint32_t x0, uint32_t y0,
                     uint32_t x1, uint32_t y1, const float* dl_di, double* grad_out, int nthreads) {
    Scene* sc = (Scene*)s;
    Camera c = cam_from(cam);
    const uint32_t cw = x1 - x0, ch = y1 - y0;
    const size_t n = sc->materials.size() * 6 + (sc->has_env ? (size_t)sc->env.width * sc->env.height * 3 : 0);
    const float inv_spp = 1.0f / (float)(spp_end - spp_begin);
    std::vector<double> total(n, 0.0);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel
#endif
    {
        std::vector<double> local(n, 0.0);
        GradPath G;
        // the throughput depends on the material parameters only (texels enter
        // through emitted radiance, added directly in add_term)
        G.n = sc->materials.size() * 6;
        G.beta_d.assign(3 * G.n, 0.0);
        G.grad = &local;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 4)
#endif
        for (int64_t pix = 0; pix < (int64_t)cw * ch; ++pix) {
            const uint32_t xx = (uint32_t)(pix % cw), yy = (uint32_t)(pix / cw);
            const uint32_t x = x0 + xx, y = y0 + yy;
            V3 delta(dl_di[3 * pix] * inv_spp, dl_di[3 * pix + 1] * inv_spp, dl_di[3 * pix + 2] * inv_spp);
            if (delta == V3()) continue;
            for (uint32_t sidx = spp_begin; sidx < spp_end; ++sidx) {
                Sampler sampler(pixel_seed(x, y, sidx));
                float jx = sampler.next_f32(), jy = sampler.next_f32();
                V2 ndc;
                ndc.x = 2.0f * ((float)x + jx) / (float)width - 1.0f;
                ndc.y = 1.0f - 2.0f * ((float)y + jy) / (float)height;
                V2 lens = sampler.next_vec2();
                float time = sampler.next_f32();
                Ray ray = c.generate_ray(ndc, lens, time);
                integrate_grad(ray, *sc, sampler, max_depth, min_rr_depth, delta, G);
            }
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        for (size_t k = 0; k < n; ++k) total[k] += local[k];
    }
    for (size_t k = 0; k < n; ++k) grad_out[k] = total[k];
}

// Single sample for path-level debugging.
void orc_render_one(void* s, const float* cam, uint32_t width, uint32_t height, uint32_t x, uint32_t y, uint32_t sidx,
                    uint32_t max_depth, uint32_t min_rr_depth, float* out10) {
    Scene* sc = (Scene*)s; Camera c = cam_from(cam);
    PixelSample ps = render_sample(*sc, c, width, height, x, y, sidx, max_depth, min_rr_depth, nullptr);
    out10[0] = ps.radiance.x; out10[1] = ps.radiance.y; out10[2] = ps.radiance.z;
    out10[3] = ps.albedo.x; out10[4] = ps.albedo.y; out10[5] = ps.albedo.z;
    out10[6] = ps.normal.x; out10[7] = ps.normal.y; out10[8] = ps.normal.z; out10[9] = ps.depth;
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
