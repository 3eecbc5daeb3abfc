// adjoint.cuh — derivatives of the BSDF value with respect to the material
// parameters (base color r,g,b, metallic, roughness, specular), in closed form
// over the same formulas as bsdf_eval (material.rs:52-58, 125-155, helpers
// 232-281), and the gradient reductions of the adjoint replay. Directions are
// not differentiated.
#pragma once
#include "shading.cuh"

namespace pyre {

#define PYRE_NPARAM 6  // base r, g, b, metallic, roughness, specular

// Parameter Jacobian of f(wo, wi) for one material, J[c][k] = d f_c / d param_k,
// in closed form over the formulas of bsdf_eval (material.rs:52-58, 125-155,
// helpers 232-281). With kd = (1-m)/pi fd_v fd_l, fd = 1 + (fd90-1) p5(cos),
// fd90 = 0.5 + 2 r cos_d^2, DG = D G / (4 cos_o cos_i), F_c = f0_c (1-p5) + p5
// and f0_c = 0.08 s (1-m) + base_c m:
//   d/d base_c   = kd + m (1-p5) DG                      (diagonal in c)
//   d/d m        = -base_c fd_v fd_l / pi + (base_c - 0.08 s)(1-p5) DG
//   d/d r        = base_c (1-m)/pi 2 cos_d^2 (p5_o fd_l + fd_v p5_i)
//                  + F_c / (4 cos_o cos_i) (dD/da2 G + D dG/da2) da2/dr
//   d/d s        = 0.08 (1-m)(1-p5) DG
// with a2 = alpha^2, alpha = max(r^2, 1e-3), dD/da2 = (den - 2 a2 hz^2) / (pi den^3)
// for den = (a2-1) hz^2 + 1, dG/da2 = -G^2 (dL_o + dL_i) and
// dL/da2 = tan2 / (4 sqrt(1 + a2 tan2)). About a sixth of the arithmetic of
// carrying six dual-number tangents through the same formulas, and the
// same speed on the adjoint replay (measured), with a smaller code footprint.
// Not inlined: it is called from several sites of a large kernel, and one
// out-of-line copy keeps the instruction footprint small.
static __device__ __noinline__ void bsdf_eval_jac(const Bsdf& b, f3 wo, f3 wi, float J[3][PYRE_NPARAM]) {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int k = 0; k < PYRE_NPARAM; ++k) J[c][k] = 0.0f;
    if (wo.z <= 0.0f || wi.z <= 0.0f) return;
    if (b.kind == PYRE_MAT_LAMBERTIAN) {  // f = albedo / pi
        J[0][0] = J[1][1] = J[2][2] = 1.0f / PYRE_PI;
        return;
    }
    const f3 h = normalize_or_zero3(wo + wi);
    if (len2(h) < 1e-10f) return;
    const float base[3] = {b.base.x, b.base.y, b.base.z};
    const float m = b.metallic, r = b.roughness, sp = b.specular;
    if (!(m >= 1.0f)) {  // diffuse (material.rs:125-138)
        const float cos_d = clampf_(dot3(wi, h), 0.0f, 1.0f);
        const float c2 = cos_d * cos_d;
        const float fd90 = 0.5f + r * (2.0f * c2);
        const float pv = powi5(fmaxf(1.0f - wo.z, 0.0f)), pl = powi5(fmaxf(1.0f - wi.z, 0.0f));
        const float fd_v = 1.0f + (fd90 - 1.0f) * pv, fd_l = 1.0f + (fd90 - 1.0f) * pl;
        const float vl = fd_v * fd_l * (1.0f / PYRE_PI);
        const float kd = (1.0f - m) * vl;
        const float kr = (1.0f - m) * (1.0f / PYRE_PI) * (2.0f * c2) * (pv * fd_l + fd_v * pl);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            J[c][c] = kd;
            J[c][3] = -base[c] * vl;
            J[c][4] = base[c] * kr;
        }
    }
    if (h.z <= 0.0f) return;
    // specular (material.rs:142-155)
    const float r2 = r * r;
    const bool clamped = !(r2 >= 1e-3f);
    const float alpha = clamped ? 1e-3f : r2;
    const float a2 = alpha * alpha;
    const float da2_dr = clamped ? 0.0f : 2.0f * alpha * (2.0f * r);
    const float hz2 = h.z * h.z;
    const float den = (a2 - 1.0f) * hz2 + 1.0f;
    const float d = a2 / ((den * den) * PYRE_PI);
    const float dd = (den - 2.0f * a2 * hz2) / (PYRE_PI * den * den * den);
    float lam_sum = 0.0f, dlam_sum = 0.0f;
    const f3 v2[2] = {wo, wi};
#pragma unroll
    for (int q = 0; q < 2; ++q) {
        const float cos2 = v2[q].z * v2[q].z;
        if (cos2 >= 1.0f) continue;
        const float tan2 = (1.0f - cos2) / fmaxf(cos2, 1e-8f);
        const float root = sqrtf(1.0f + a2 * tan2);
        lam_sum += 0.5f * (root - 1.0f);
        dlam_sum += root > 0.0f ? 0.25f * tan2 / root : 0.0f;
    }
    const float g = 1.0f / (1.0f + lam_sum);
    const float dg = -g * g * dlam_sum;
    const float cd = clampf_(fmaxf(dot3(wi, h), 0.0f), 0.0f, 1.0f);
    const float p5 = powi5(1.0f - cd);
    const float inv = 1.0f / (4.0f * wo.z * wi.z);
    const float dgi = d * g * inv;                          // D G / (4 cos_o cos_i)
    const float dr_s = (dd * g + d * dg) * inv * da2_dr;    // d(D G / (4 cos cos)) / d r
    const float diel = 0.08f * sp;
    const float q5 = 1.0f - p5;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const float f0 = diel * (1.0f - m) + base[c] * m;
        const float F = f0 + (1.0f - f0) * p5;
        J[c][c] += m * q5 * dgi;
        J[c][3] += (base[c] - diel) * q5 * dgi;
        J[c][4] += F * dr_s;
        J[c][5] = 0.08f * (1.0f - m) * q5 * dgi;
    }
}

// The four texels and weights of env_texture's bilinear lookup (light.rs:290-314).
__device__ __forceinline__ void env_texel_weights(const DevEnv& E, f2 uv, uint32_t idx[4], float wt[4]) {
    int32_t w = (int32_t)E.width, h = (int32_t)E.height;
    float u = fract_(fract_(uv.x) + 1.0f);
    float v = clampf_(uv.y, 0.0f, 1.0f);
    float fx = u * (float)w - 0.5f;
    float fy = clampf_(v * (float)h - 0.5f, 0.0f, (float)h - 1.0f);
    int32_t x0i = sat_i32(floorf(fx)), y0i = sat_i32(floorf(fy));
    float dx = fx - (float)x0i, dy = fy - (float)y0i;
    int32_t x0 = ((x0i % w) + w) % w;
    int32_t x1 = ((x0 + 1) % w + w) % w;
    int32_t y0 = min(max(y0i, 0), h - 1);
    int32_t y1 = min(y0 + 1, h - 1);
    idx[0] = (uint32_t)(y0 * w + x0); wt[0] = (1.0f - dx) * (1.0f - dy);
    idx[1] = (uint32_t)(y0 * w + x1); wt[1] = dx * (1.0f - dy);
    idx[2] = (uint32_t)(y1 * w + x0); wt[2] = (1.0f - dx) * dy;
    idx[3] = (uint32_t)(y1 * w + x1); wt[3] = dx * dy;
}

// Warp aggregation of the gradient atomics. The lanes of a warp (those
// converged here) that add to the same address first sum their terms, and
// one lane adds the sum. Many paths share a material, and importance
// sampling sends most environment samples to the few texels of a bright
// lobe, so one atomic per term serializes on those addresses.
//
// peer_sum: the sum of v over the lanes in `peers`; every lane of `peers`
// calls it with the same mask. The leader's value is the one used.
template <class T>
__device__ __forceinline__ T peer_sum(unsigned peers, T v) {
    if ((peers & (peers - 1u)) == 0u) return v;  // alone
    if (peers == 0xffffffffu) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        return v;
    }
    T s = T(0);
    for (unsigned rest = peers; rest; rest &= rest - 1) s += __shfl_sync(peers, v, __ffs(rest) - 1);
    return s;
}

// Full-warp sum of v (all 32 lanes call it).
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

#define PYRE_NO_KEY 0xffffffffu

// Texel gradients of one block go through a cache in shared memory: a
// direct-mapped table of PYRE_ENV_CACHE slots, each claimed for good by the
// first texel that hashes to it and summed with shared-memory atomics; the
// block adds the table to the gradient once, when it ends. Importance
// sampling sends most environment terms to the few texels of a bright lobe,
// and one global atomic per term (even after warp aggregation) queued on
// those addresses. A texel whose slot another texel holds adds directly.
#ifndef PYRE_ENV_CACHE_LOG2
#define PYRE_ENV_CACHE_LOG2 10  // 1024 slots, 20 KB of shared memory per block
#endif
#define PYRE_ENV_CACHE (1u << PYRE_ENV_CACHE_LOG2)
// With the cache, each lane adds its texel terms to it directly: the warp's
// butterflies cost more than shared-memory atomics on a shared slot. The
// backward of the 512^2 problem took 24.6 against 27.4 ms (27.4 with warp
// aggregation and no cache).
#ifndef PYRE_ENV_CACHE_DIRECT
#define PYRE_ENV_CACHE_DIRECT 1
#endif
// Material terms: lanes that hold the same material (most of a warp once the
// backward sorts its paths by material) are summed with full-warp FP32
// butterflies, and one lane adds each sum to the block's FP64 sums in shared
// memory; other lanes add their own terms. The backward of the 512^2 problem
// took 19.3 ms, against 19.7 with FP64 butterflies and 20.0 with every lane
// adding to the FP64 sums (PYRE_MAT_DIRECT; before the material sort that
// was the fastest: 23.9 against 24.6 ms). A warp sums at most 32 terms in
// FP32; the sums over the block and the image stay FP64.
#ifndef PYRE_MAT_WARP32
#define PYRE_MAT_WARP32 1
#endif
#ifndef PYRE_MAT_DIRECT
#define PYRE_MAT_DIRECT 0
#endif

// A block's gradient accumulators in its dynamic shared memory: the texel
// cache (null without texel gradients), then the material sums (null when
// they add to global memory directly).
struct GradSmem {
    float4* cval;    // PYRE_ENV_CACHE texel sums (x, y, z)
    uint32_t* ckey;  // the texel of each slot, PYRE_NO_KEY while free
    double* mat;     // n_mat * PYRE_NPARAM material sums
};

// Bytes of dynamic shared memory for the accumulators.
__host__ __device__ __forceinline__ size_t grad_smem_bytes(bool env_cache, size_t mat_bytes) {
    return (env_cache ? (size_t)PYRE_ENV_CACHE * (sizeof(float4) + sizeof(uint32_t)) : 0) + mat_bytes;
}

// Lays out and clears the block's accumulators (all threads of the block call it).
__device__ __forceinline__ GradSmem grad_smem_begin(bool env_cache, bool mat_smem, uint32_t n_mat) {
    extern __shared__ float4 grad_dyn_smem[];
    GradSmem G;
    char* p = reinterpret_cast<char*>(grad_dyn_smem);
    G.cval = nullptr; G.ckey = nullptr; G.mat = nullptr;
    if (env_cache) {
        G.cval = reinterpret_cast<float4*>(p);
        G.ckey = reinterpret_cast<uint32_t*>(p + PYRE_ENV_CACHE * sizeof(float4));
        p += PYRE_ENV_CACHE * (sizeof(float4) + sizeof(uint32_t));
        for (uint32_t k = threadIdx.x; k < PYRE_ENV_CACHE; k += blockDim.x) {
            G.cval[k] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            G.ckey[k] = PYRE_NO_KEY;
        }
    }
    if (mat_smem) {
        G.mat = reinterpret_cast<double*>(p);
        for (uint32_t k = threadIdx.x; k < n_mat * PYRE_NPARAM; k += blockDim.x) G.mat[k] = 0.0;
    }
    __syncthreads();
    return G;
}

// Adds the block's accumulators to the gradients (all threads of the block call it).
__device__ __forceinline__ void grad_smem_end(const GradSmem& G, float* env_grad, double* mat_grad, uint32_t n_mat) {
    if (!G.cval && !G.mat) return;
    __syncthreads();
    if (G.cval)
        for (uint32_t k = threadIdx.x; k < PYRE_ENV_CACHE; k += blockDim.x) {
            const uint32_t t = G.ckey[k];
            if (t == PYRE_NO_KEY) continue;
            const float4 v = G.cval[k];
            if (v.x != 0.0f) atomicAdd(env_grad + 3 * (size_t)t, v.x);
            if (v.y != 0.0f) atomicAdd(env_grad + 3 * (size_t)t + 1, v.y);
            if (v.z != 0.0f) atomicAdd(env_grad + 3 * (size_t)t + 2, v.z);
        }
    if (G.mat)
        for (uint32_t k = threadIdx.x; k < n_mat * PYRE_NPARAM; k += blockDim.x)
            if (G.mat[k] != 0.0) atomicAdd(mat_grad + k, G.mat[k]);
}

// d(loss)/d(texel t) += (x, y, z), through the block's cache when it has one.
__device__ __forceinline__ void env_grad_add(float* env_grad, const GradSmem& G, uint32_t t, float x, float y,
                                             float z) {
    if (G.ckey) {
        const uint32_t slot = (t * 2654435761u) >> (32 - PYRE_ENV_CACHE_LOG2);
        uint32_t k = *reinterpret_cast<volatile uint32_t*>(G.ckey + slot);
        if (k == PYRE_NO_KEY) {
            const uint32_t old = atomicCAS(G.ckey + slot, PYRE_NO_KEY, t);
            k = old == PYRE_NO_KEY ? t : old;
        }
        if (k == t) {
            float* v = reinterpret_cast<float*>(G.cval + slot);
            if (x != 0.0f) atomicAdd(v, x);
            if (y != 0.0f) atomicAdd(v + 1, y);
            if (z != 0.0f) atomicAdd(v + 2, z);
            return;
        }
    }
    const size_t a = 3 * (size_t)t;
    if (x != 0.0f) atomicAdd(env_grad + a, x);
    if (y != 0.0f) atomicAdd(env_grad + a + 1, y);
    if (z != 0.0f) atomicAdd(env_grad + a + 2, z);
}

// d(loss)/d(texel) for a radiance term c * Le(uv), Le = texture(uv) * intensity.
__device__ __forceinline__ void scatter_env(const DevEnv& E, float* env_grad, const GradSmem& G, f2 uv, f3 c) {
    if (!env_grad) return;
    uint32_t idx[4];
    float wt[4];
    env_texel_weights(E, uv, idx, wt);
#if PYRE_ENV_CACHE_DIRECT
    if (G.ckey) {
        for (int k = 0; k < 4; ++k) {
            const float s = wt[k] * E.intensity;
            if (s != 0.0f) env_grad_add(env_grad, G, idx[k], c.x * s, c.y * s, c.z * s);
        }
        return;
    }
#endif
    const unsigned act = __activemask();
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float s = wt[k] * E.intensity;
        const uint32_t key = s != 0.0f ? idx[k] : 0xffffffffu;  // zero weights add nothing
        const unsigned peers = __match_any_sync(act, key);
        const float x = peer_sum(peers, c.x * s), y = peer_sum(peers, c.y * s), z = peer_sum(peers, c.z * s);
        if (key == 0xffffffffu || lane != __ffs(peers) - 1) continue;
        env_grad_add(env_grad, G, key, x, y, z);
    }
}

}  // namespace pyre

namespace pyre {

#define PYRE_FLUSH_ROUNDS 3  // keys aggregated per flush; the rest add directly

// One lane's gradient terms of one path vertex, added at a point where the
// warp is converged (warp_flush): the 6 parameters of one material (all the
// terms of a vertex belong to the material of the previous vertex), and one
// environment footprint (c, added to the 4 texels of uv's bilinear lookup).
struct GradTerms {
    uint32_t mat = PYRE_NO_KEY;
    float g[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    bool env = false;
    f2 uv;
    f3 c;
};

// Adds every lane's terms. With all 32 lanes converged, the lanes holding the
// same material (or the same footprint) are summed with full-warp butterflies
// (FP64 for materials), for up to PYRE_FLUSH_ROUNDS keys per kind that more
// than one lane holds, and one lane adds each sum; every other lane adds its
// own terms. A warp that is not converged adds lane by lane.
__device__ __forceinline__ void warp_flush(const DevScene& S, float* env_grad, double* mat_grad, const GradSmem& G,
                                           const GradTerms& t) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    bool full = __activemask() == FULL;
    auto mat_add = [&](uint32_t m, int k, double v) {
        if (v == 0.0) return;
        if (G.mat) atomicAdd(G.mat + PYRE_NPARAM * m + k, v);
        else atomicAdd(mat_grad + PYRE_NPARAM * (size_t)m + k, v);
    };
    // materials
    bool left = t.mat != PYRE_NO_KEY;
#if PYRE_MAT_DIRECT
    if (G.mat) {  // the block's FP64 sums in shared memory take each lane's terms directly
        if (left)
            for (int k = 0; k < PYRE_NPARAM; ++k) mat_add(t.mat, k, (double)t.g[k]);
        left = false;
    }
#endif
    if (full && __any_sync(FULL, left)) {
        // only keys that several lanes hold are worth a butterfly
        const unsigned peers = __match_any_sync(FULL, t.mat);
        unsigned todo = __ballot_sync(FULL, left && (peers & (peers - 1u)) != 0u);
        for (int r = 0; r < PYRE_FLUSH_ROUNDS && todo; ++r) {
            const int src = __ffs(todo) - 1;
            const uint32_t key = __shfl_sync(FULL, t.mat, src);
            const bool mine = left && t.mat == key;
            todo &= ~__ballot_sync(FULL, mine);
#pragma unroll
            for (int k = 0; k < PYRE_NPARAM; ++k) {
#if PYRE_MAT_WARP32
                const double v = (double)warp_sum(mine ? t.g[k] : 0.0f);
#else
                const double v = warp_sum(mine ? (double)t.g[k] : 0.0);
#endif
                if (lane == src) mat_add(key, k, v);
            }
            if (mine) left = false;
        }
    }
    if (left)
        for (int k = 0; k < PYRE_NPARAM; ++k) mat_add(t.mat, k, (double)t.g[k]);
    // environment footprint
    if (!env_grad) return;
    uint32_t idx[4];
    float wt[4];
    f3 c = splat3(0.0f);
    uint32_t key = PYRE_NO_KEY;
    if (t.env) {
        env_texel_weights(S.env, t.uv, idx, wt);
        key = idx[0];  // the other three texels follow from the first
        c = t.c * S.env.intensity;
    }
    left = key != PYRE_NO_KEY;
#if PYRE_ENV_CACHE_DIRECT
    // with the block's cache the lanes add their own terms: shared-memory
    // atomics on one slot cost less than the warp's butterflies
    if (G.ckey) full = false;
#endif
    if (full) {
        const unsigned peers = __match_any_sync(FULL, key);
        unsigned todo = __ballot_sync(FULL, left && (peers & (peers - 1u)) != 0u);
        for (int r = 0; r < PYRE_FLUSH_ROUNDS && todo; ++r) {
            const int src = __ffs(todo) - 1;
            const uint32_t k0 = __shfl_sync(FULL, key, src);
            const bool mine = left && key == k0;
            todo &= ~__ballot_sync(FULL, mine);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float x = warp_sum(mine ? c.x * wt[q] : 0.0f), y = warp_sum(mine ? c.y * wt[q] : 0.0f),
                            z = warp_sum(mine ? c.z * wt[q] : 0.0f);
                if (lane == src) env_grad_add(env_grad, G, idx[q], x, y, z);
            }
            if (mine) left = false;
        }
    }
    if (left)
        for (int q = 0; q < 4; ++q) {
            if (wt[q] == 0.0f) continue;
            env_grad_add(env_grad, G, idx[q], c.x * wt[q], c.y * wt[q], c.z * wt[q]);
        }
}

}  // namespace pyre
