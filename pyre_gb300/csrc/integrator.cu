// integrator.cu — wavefront path tracer and ray-query kernels for sm_103a.
//
// One render = waves of paths. A wave holds K samples of every pixel of the
// crop (path i -> sample s_base + i / npix, pixel i % npix), so the film can
// sum sample radiance in the same order as the CLI loop
// (crates/pyre-cli/src/main.rs:260-285). Each wave runs
//   raygen -> [extend -> shade -> shadow] x max_depth -> accumulate
// over structure-of-arrays path state in HBM, with the live paths and the
// shadow rays kept in compacted queues (warp-aggregated appends). Every path
// carries its own Xoshiro256++ state, so the sampler draws happen in the
// reference's order: jitter x/y, lens x/y, time at raygen; then per surface
// vertex one vec2 per quad light, one vec2 for the environment, one vec2 for
// the BSDF sample and one f32 for Russian roulette (integrator.rs:307-375).
// NEE contributions are computed at shade time assuming visibility and parked
// in per-path slots; the shadow stage clears the slot of an occluded ray; the
// next shade (or the accumulate stage) adds the surviving slots in light
// order, which is the reference's summation order.
#include <cooperative_groups.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "internal.h"
#include "adjoint.cuh"
#include "shading.cuh"

namespace cg = cooperative_groups;

namespace pyre {

#define PYRE_MAX_DEPTH 64
// resident blocks of 128 threads per SM for closest-hit (extend, ray queries) and any-hit (shadow) traversal
// (with instances entered from the top-level step, 9 closest-hit blocks
// measured 746.2 against 737.9 Msamples/s for 10 and 743.4 for 8; any hit at
// 10 blocks took 36.0 against 34.5 ms of shadow)
// forward shade: threads per block and resident blocks per SM. With the
// material-sorted queue, 224 x 4 (72 registers) measured 784.2 Msamples/s on
// the 1080p studio frame, 192 x 5 782.9, 128 x 7 781.6 and 256 x 3 757.7.
#ifndef PYRE_SHADE_THREADS
#define PYRE_SHADE_THREADS 224
#endif
#ifndef PYRE_SHADE_BLOCKS
#define PYRE_SHADE_BLOCKS 4
#endif
#ifndef PYRE_TRACE_BLOCKS
#define PYRE_TRACE_BLOCKS 9
#endif
#ifndef PYRE_TRACE_BLOCKS_ANY
#define PYRE_TRACE_BLOCKS_ANY 9
#endif
#define PYRE_SORT_BINS 1024  // shade-queue sort keys: escaped, light hit, then materials
// WaveParams::sort: how shade's queue is ordered by material
#define PYRE_SORT_OFF 0
#define PYRE_SORT_TILES 1  // within tiles of PYRE_SORT_TILE_N consecutive entries
#define PYRE_SORT_QUEUE 2  // the whole queue

struct WaveCtl {
    uint32_t wave;
    uint32_t s_base;
    uint32_t k_valid;
    uint32_t n_valid;
    uint32_t count[PYRE_MAX_DEPTH + 1];   // extend queue sizes per depth
    uint32_t scount[PYRE_MAX_DEPTH];      // shadow queue sizes per depth
    uint32_t fetch[2 * PYRE_MAX_DEPTH];   // work counters of extend / shadow
    unsigned long long extend_rays, shadow_rays, samples;
    // material sort of the shade queue: bin sizes (zero between sorts) and bin offsets
    uint32_t sort_hist[PYRE_SORT_BINS];
    uint32_t sort_off[PYRE_SORT_BINS];
};

// Batched rendering: per-job view, per-wave segments (a segment = one job's
// consecutive samples s_first .. s_first+s_count-1 over all its pixels).
struct DevJob {
    DevCamera cam;
    uint32_t width, height, npix;
    uint32_t spp_begin, spp_end, max_depth, min_rr;
    int32_t tlas_root;
    uint32_t light_first, light_count;
    uint32_t acc_base;  // first film accumulator of the job
    float inv_spp;
};
struct DevSeg {
    uint32_t job, s_first, s_count;
    uint32_t path_base;  // first path of the segment in the wave
    uint32_t slot_base;  // first accumulate slot (one per pixel) of the segment
};
struct DevWave {
    uint32_t seg_first, seg_count;
    uint32_t n_paths, n_slots;
};

struct WaveParams {
    DevCamera cam;
    uint32_t width, height;
    uint32_t cx0, cy0, cw, ch, npix;
    uint32_t spp_begin, spp_end, k_per_wave;
    uint32_t max_depth, min_rr;
    uint32_t ns;  // NEE slots per path: lights (+1 for the environment)
    int env_cdf;
    // batch tables (null for a single view)
    const DevJob* jobs;
    const DevSeg* segs;
    const DevWave* waves;
    // adjoint replay
    const float* dl_di;  // crop npix*3: d loss / d film radiance
    float inv_spp;
    double* mat_grad;    // n_mat*6
    float* env_grad;     // env texels*3 or null
    uint32_t n_mat;
    int smem_grad;       // material gradients summed per block in shared memory
    int env_cache;       // texel gradients summed per block through a shared-memory cache
    int refill;          // traversal: idle lanes of a warp that trigger a refetch (closest hit)
    int refill_any;      // the same for the any-hit (shadow) traversal
    int sort;            // shade reads the live paths sorted by material (P.qsort)
    int bvh_width;       // instance BVH width of the traversal kernels: 2, 4 or 8
    // progressive accumulation (pyre_render_progressive): crop npix x 3 running
    // mean of the radiance, updated once per sample in sample order
    float* prog_mean;
};

// Default ray-refill thresholds (idle lanes of a warp) of closest-hit and
// any-hit traversal; a nonzero refill_lanes sets both. Closest hit at 12
// (with lanes that stop at their first leaf and the leaf phase at 16 seeking
// lanes): 762.3 against 758.8 Msamples/s for 16 and 755.2 for 20 on the
// 1080p studio frame; microbenchmark closest hit 3.75 against 4.01 ms.
#ifndef PYRE_DEFAULT_REFILL
#define PYRE_DEFAULT_REFILL 12
#endif
#ifndef PYRE_DEFAULT_REFILL_ANY
#define PYRE_DEFAULT_REFILL_ANY 8
#endif
static inline int refill_lanes(const pyre_render_params* rp, bool any_hit = false) {
    const uint32_t v = rp ? rp->refill_lanes : 0u;
    if (v == 0) return any_hit ? PYRE_DEFAULT_REFILL_ANY : PYRE_DEFAULT_REFILL;
    return (int)std::min<uint32_t>(v, 32u);
}

// sort_by_material of pyre_render_params: 0 = the call's default, 1 = within
// tiles, 2 = off, 3 = the whole queue; -1 for any other value.
int sort_kind(uint32_t v, int dflt) {
    switch (v) {
        case 0: return dflt;
        case 1: return PYRE_SORT_TILES;
        case 2: return PYRE_SORT_OFF;
        case 3: return PYRE_SORT_QUEUE;
        default: return -1;
    }
}

#define PYRE_GSLOT 4  // float4s of parked gradient terms per NEE slot

struct PathSoA {
    // rays and hits live at queue positions: entry j of the depth's live-path
    // queue (at depth 0, the path index). Depth d reads ray_o/ray_d[d & 1];
    // shade writes the next depth's rays into the other buffer.
    float4* ray_o[2];  // origin.xyz
    float4* ray_d[2];  // direction.xyz, time
    float4* hit;       // t, u, v, triangle slot (bits)
    int32_t* hit_inst; // instance slot; -1 miss; -2-l quad light l
    uint4* rng;        // 2 per path
    float4* Lb;        // 2 per path, one 32-B record: radiance.xyz, -; throughput.xyz, pdf of the
                       // last BSDF sample (shade reads and writes both with one access each)
    float4* aov;       // 2 per path, one 32-B record: albedo.xyz, depth; normal.xyz, -
    float4* pend;      // ns per path: NEE contribution.xyz, w = 1 while pending
    float4* sh_o;      // per shadow-queue entry: shadow origin.xyz, t_max
    float4* sh_d;      // per shadow-queue entry: shadow direction.xyz, time
    uint32_t* q[2];
    uint32_t* qsort;   // the live paths of the current depth ordered by shade_key
    uint32_t* sq;
    float4* acc_r;     // per crop pixel: radiance sum.xyz, depth sum
    float4* acc_a;     // albedo sum
    float4* acc_n;     // normal sum
    WaveCtl* ctl;
    int32_t* sroot;    // batch: per shadow-queue entry, the top-level root of the ray's job
    // adjoint replay (null otherwise)
    float4* keep_L;    // per (sample, pixel) of the sample range: final path radiance (pyre_forward)
    float4* gpend;     // 3 per NEE slot: parked gradient terms of that slot
    float4* brec;      // 3 per path: BSDF sample of the last vertex (wo+mat, wi+flag, f)
};

__device__ __forceinline__ uint32_t append_slot(uint32_t* counter) {
    cg::coalesced_group g = cg::coalesced_threads();
    uint32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(counter, g.size());
    base = g.shfl(base, 0);
    return base + g.thread_rank();
}

// A path's generator state is one 32-B record: one 256-bit access each way.
__device__ __forceinline__ void store_rng(uint4* r, uint32_t i, const Rng& g) {
    auto f = [](uint64_t v, int hi) { return __uint_as_float((uint32_t)(hi ? v >> 32 : v)); };
    stcs_256(reinterpret_cast<float4*>(r + 2 * (size_t)i),
             make_float4(f(g.s0, 0), f(g.s0, 1), f(g.s1, 0), f(g.s1, 1)),
             make_float4(f(g.s2, 0), f(g.s2, 1), f(g.s3, 0), f(g.s3, 1)));
}
__device__ __forceinline__ Rng load_rng(const uint4* r, uint32_t i) {
    float4 a, b;
    ldcs_256(reinterpret_cast<const float4*>(r + 2 * (size_t)i), a, b);
    auto u = [](float lo, float hi) { return (uint64_t)__float_as_uint(lo) | ((uint64_t)__float_as_uint(hi) << 32); };
    Rng g;
    g.s0 = u(a.x, a.y);
    g.s1 = u(a.z, a.w);
    g.s2 = u(b.x, b.y);
    g.s3 = u(b.z, b.w);
    return g;
}

// ------------------------------------------------------------------ wave --
__global__ void k_wave_begin(WaveCtl* ctl, uint32_t spp_begin, uint32_t spp_end, uint32_t K, uint32_t npix) {
    if (threadIdx.x != 0) return;
    uint32_t s_base = spp_begin + ctl->wave * K;
    uint32_t k_valid = s_base < spp_end ? min(K, spp_end - s_base) : 0u;
    ctl->s_base = s_base;
    ctl->k_valid = k_valid;
    ctl->n_valid = k_valid * npix;
    for (int d = 0; d <= PYRE_MAX_DEPTH; ++d) ctl->count[d] = 0;
    for (int d = 0; d < PYRE_MAX_DEPTH; ++d) ctl->scount[d] = 0;
    for (int d = 0; d < 2 * PYRE_MAX_DEPTH; ++d) ctl->fetch[d] = 0;
    ctl->count[0] = k_valid * npix;
}

__global__ void k_wave_begin_batch(WaveCtl* ctl, const DevWave* waves) {
    if (threadIdx.x != 0) return;
    const DevWave w = waves[ctl->wave];
    ctl->s_base = 0;
    ctl->k_valid = 0;
    ctl->n_valid = w.n_paths;
    for (int d = 0; d <= PYRE_MAX_DEPTH; ++d) ctl->count[d] = 0;
    for (int d = 0; d < PYRE_MAX_DEPTH; ++d) ctl->scount[d] = 0;
    for (int d = 0; d < 2 * PYRE_MAX_DEPTH; ++d) ctl->fetch[d] = 0;
    ctl->count[0] = w.n_paths;
}

// Segment of the current wave holding path (or slot) i: last segment whose
// base is <= i (binary search over the wave's segments).
__device__ __forceinline__ uint32_t find_segment(const DevSeg* segs, const DevWave& w, uint32_t i, bool by_slot) {
    uint32_t lo = w.seg_first, hi = w.seg_first + w.seg_count - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi + 1) / 2;
        uint32_t b = by_slot ? segs[mid].slot_base : segs[mid].path_base;
        if (b <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__global__ void k_wave_end(WaveCtl* ctl, uint32_t max_depth) {
    if (threadIdx.x != 0) return;
    unsigned long long e = 0, s = 0;
    for (uint32_t d = 0; d < max_depth; ++d) { e += ctl->count[d]; s += ctl->scount[d]; }
    ctl->extend_rays += e;
    ctl->shadow_rays += s;
    ctl->samples += ctl->n_valid;
    ctl->wave += 1;
}

// main.rs:261-273: seed, jitter, ndc, lens, time, Camera::generate_ray.
template <bool BATCH>
__global__ void k_raygen(PathSoA P, WaveParams W) {
    const uint32_t n = P.ctl->n_valid;
    const uint32_t s_base = P.ctl->s_base;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t x, y, s, width, height, max_depth = W.max_depth, job = 0;
        const DevCamera* cam = &W.cam;
        if (BATCH) {
            const DevWave& wv = W.waves[P.ctl->wave];
            const DevSeg sg = W.segs[find_segment(W.segs, wv, i, false)];
            const DevJob& J = W.jobs[sg.job];
            const uint32_t local = i - sg.path_base, k = local / J.npix, p = local - k * J.npix;
            x = p % J.width; y = p / J.width; s = sg.s_first + k;
            width = J.width; height = J.height;
            max_depth = J.max_depth;
            cam = &J.cam;
            job = sg.job;
        } else {
            const uint32_t k = i / W.npix, p = i - k * W.npix;
            x = W.cx0 + p % W.cw; y = W.cy0 + p / W.cw; s = s_base + k;
            width = W.width; height = W.height;
        }
        Rng g;
        g.seed(pixel_seed(x, y, s));
        float jx = g.next_f32(), jy = g.next_f32();
        f2 ndc;
        ndc.x = 2.0f * ((float)x + jx) / (float)width - 1.0f;
        ndc.y = 1.0f - 2.0f * ((float)y + jy) / (float)height;
        f2 lens = g.next_vec2();
        float time = g.next_f32();
        f3 o, d;
        camera_ray(*cam, ndc, lens, &o, &d);
        // a batch ray carries its job in the origin's w (the traversal's t_min is a constant)
        __stcs(&P.ray_o[0][i], make_float4(o.x, o.y, o.z, BATCH ? __uint_as_float(job) : 1e-4f));
        __stcs(&P.ray_d[0][i], make_float4(d.x, d.y, d.z, time));
        store_rng(P.rng, i, g);
        // radiance 0, throughput 1 and the AOVs are set by shade at depth 0;
        // with max_depth 0 no vertex is shaded and the sample is all zeros
        if (max_depth == 0) {
            P.Lb[2 * (size_t)i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            stcs_256(P.aov + 2 * (size_t)i, make_float4(0.0f, 0.0f, 0.0f, 0.0f), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        }
        for (uint32_t s = 0; s < W.ns; ++s) __stcs(P.pend + (size_t)i * W.ns + s, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    }
}

// Depth-0 order of a single view's wave: extend and shade take the camera
// paths in 8x4 pixel tiles, so a warp's 32 rays cover a compact footprint
// instead of 32 pixels of one row. j -> path index k * npix + p is a
// bijection of [0, k_valid * npix): tiles run along bands of 4 crop rows (the
// last band may be shorter), and a band's last cw % 8 columns are taken row by
// row. Path indices, seeds and the film's sample order stay row-major.
#define PYRE_TILE_W 8u
#define PYRE_TILE_H 4u
__device__ __forceinline__ uint32_t tiled_path(const WaveParams& W, uint32_t j) {
    const uint32_t k = j / W.npix, q = j - k * W.npix;
    const uint32_t band_px = W.cw * PYRE_TILE_H, full_bands = W.ch / PYRE_TILE_H;
    uint32_t band = q / band_px, hb = PYRE_TILE_H;
    if (band >= full_bands) { band = full_bands; hb = W.ch - full_bands * PYRE_TILE_H; }
    const uint32_t r = q - band * band_px;
    const uint32_t cwt = W.cw - W.cw % PYRE_TILE_W;  // columns in whole tiles
    uint32_t x, y;
    if (r < hb * cwt) {
        const uint32_t tile_px = PYRE_TILE_W * hb, c = r / tile_px, l = r - c * tile_px;
        x = c * PYRE_TILE_W + l % PYRE_TILE_W;
        y = l / PYRE_TILE_W;
    } else {
        const uint32_t rw = W.cw - cwt, rem = r - hb * cwt;
        x = cwt + rem % rw;
        y = rem / rw;
    }
    return k * W.npix + (band * PYRE_TILE_H + y) * W.cw + x;
}

// ---------------------------------------------------------------- extend --
// Path state is read and written once per stage through the live-path
// queues, so the traversal and shade kernels access it with streaming cache
// hints (__ldcs / __stcs, evict-first); the scene's nodes and triangles keep
// the L2 (+1.2 % on the 1080p studio frame for the loads and hit stores,
// +0.35 % more for shade's stores).
// Closest hit of the live paths (Scene::intersect, scene.rs:57-97).
template <bool BATCH>
struct ExtendRays {
    // every extend ray has this t range (the traversal's idle lanes start
    // with it too, so the compiler keeps it out of registers: spills 16
    // against 28 B, 811.4 against 802.4 Msamples/s on the 1080p studio frame)
    static constexpr float kTmin = 1e-4f, kTmax = INFINITY;
    const DevScene* S;
    const PathSoA* P;
    const WaveParams* W;
    const uint32_t* qin;  // live-path queue; null at depth 0 (every path of the wave)
    uint32_t depth;
    // ray j of the queue sits at queue position j (depth 0: path tiled_path(j))
    __device__ __forceinline__ uint32_t load(uint32_t j, TraceRay& r, int32_t& root) const {
        const uint32_t p = qin ? j : (BATCH ? j : tiled_path(*W, j));
        const float4 ro = __ldcs(P->ray_o[depth & 1] + p), rd = __ldcs(P->ray_d[depth & 1] + p);
        r.o = mk3(ro.x, ro.y, ro.z);
        r.d = mk3(rd.x, rd.y, rd.z);
        r.tmin = 1e-4f;
        r.tmax = __int_as_float(0x7f800000);
        r.time = rd.w;
        r.job = BATCH ? __float_as_uint(ro.w) : 0u;  // batch: the ray's job
        root = BATCH ? W->jobs[r.job].tlas_root : S->tlas_root;
        return p;
    }
    __device__ __forceinline__ void store(uint32_t p, const TraceRay& r, TraceHit& h, bool) const {
        uint32_t lfirst = 0, lcount = S->n_lights;
        if (BATCH) {
            const DevJob& J = W->jobs[r.job];
            lfirst = J.light_first; lcount = J.light_count;
        }
        hit_quad_lights(*S, r, lfirst, lcount, &h);
        __stcs(P->hit + p, make_float4(h.t, h.u, h.v, __int_as_float(h.tri)));
        __stcs(P->hit_inst + p, h.light >= 0 ? -2 - h.light : h.inst);
    }
};

// The traversal kernels are persistent grids of resident 128-thread blocks,
// 9 per SM (56 registers). Warps wait mostly on node, triangle and stack
// loads, so more of them per SM pay, up to where the spills that a smaller
// register budget forces cost more than the extra warps hide.
template <bool BATCH, int WIDTH>
__global__ void __launch_bounds__(128, PYRE_TRACE_BLOCKS) k_extend(DevScene S, PathSoA P, WaveParams W, uint32_t depth) {
    ExtendRays<BATCH> src{&S, &P, &W, depth == 0 ? nullptr : P.q[depth & 1], depth};
    trace_stream<false, WIDTH>(S, src, P.ctl->count[depth], &P.ctl->fetch[2 * depth], W.refill);
}

// ---------------------------------------------------------------- shadow --
// Visibility of the parked NEE contributions (Scene::occluded /
// occluded_dir, scene.rs:102-140): an occluded ray clears its slot.
template <bool BATCH>
struct ShadowRays {
    static constexpr float kTmin = 1e-3f, kTmax = 0.0f;  // t_min is fixed; t_max comes with each ray
    const DevScene* S;
    const PathSoA* P;
    const WaveParams* W;
    __device__ __forceinline__ uint32_t load(uint32_t j, TraceRay& r, int32_t& root) const {
        // the ray sits at its queue entry, so these loads do not wait for sq
        const uint32_t target = __ldcs(P->sq + j);
        const float4 so = __ldcs(P->sh_o + j), sd = __ldcs(P->sh_d + j);
        r.o = mk3(so.x, so.y, so.z);
        r.d = mk3(sd.x, sd.y, sd.z);
        r.tmin = 1e-3f;
        r.tmax = so.w;
        r.time = sd.w;
        root = BATCH ? __ldcs(P->sroot + j) : S->tlas_root;
        return target;
    }
    __device__ __forceinline__ void store(uint32_t target, const TraceRay&, TraceHit&, bool occluded) const {
        if (!occluded) return;
        P->pend[target] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (P->gpend) P->gpend[PYRE_GSLOT * (size_t)target + 1].w = 0.0f;  // its gradient terms die with it
    }
};

template <bool BATCH, int WIDTH>
__global__ void __launch_bounds__(128, PYRE_TRACE_BLOCKS_ANY) k_shadow(DevScene S, PathSoA P, WaveParams W, uint32_t depth) {
    ShadowRays<BATCH> src{&S, &P, &W};
    trace_stream<true, WIDTH>(S, src, P.ctl->scount[depth], &P.ctl->fetch[2 * depth + 1], W.refill_any);
}

// ------------------------------------------------------- adjoint helpers --
// d loss . (J (x) w): the parameter gradient of a term  w (x) f(wo, wi).
__device__ __forceinline__ void jac_dot(const Bsdf& b, f3 wo, f3 wi, f3 w, float g[6]) {
    float J[3][PYRE_NPARAM];
    bsdf_eval_jac(b, wo, wi, J);
#pragma unroll
    for (int k = 0; k < PYRE_NPARAM; ++k) g[k] = w.x * J[0][k] + w.y * J[1][k] + w.z * J[2][k];
}
// Collects the parked gradient terms of one visible NEE slot (layout:
// g0 = params 0-3, g1 = (params 4-5, material bits, pending), g2 = (env uv,
// env flag, -), g3 = (env texel weight rgb, -)). All slots of a vertex share
// its material, and at most one (the environment's) has a footprint.
__device__ __forceinline__ void collect_parked_grad(const float4* G, GradTerms& t) {
    const float4 g0 = G[0], g1 = G[1];
    if (g1.w == 0.0f) return;
    t.mat = __float_as_uint(g1.z);
    t.g[0] += g0.x; t.g[1] += g0.y; t.g[2] += g0.z; t.g[3] += g0.w; t.g[4] += g1.x; t.g[5] += g1.y;
    const float4 g2 = G[2];
    if (g2.z != 0.0f) {
        const float4 g3 = G[3];
        t.env = true;
        t.uv.x = g2.x; t.uv.y = g2.y;
        t.c = mk3(g3.x, g3.y, g3.z);
    }
}

// ------------------------------------------------------- material sort --
// Counting sort of the live paths by what shade will run for them: escaped
// paths, quad-light hits, then one bin per material (modulo the bin count).
// Shade then sees warps of one material, with one code path (Lambertian or
// Disney) and the same material record. Results do not depend on the order
// in which shade visits paths.
__device__ __forceinline__ uint32_t shade_key(const DevScene& S, int32_t code) {
    if (code == -1) return 0u;
    if (code <= -2) return 1u;
    return 2u + S.inst[code].material % (uint32_t)(PYRE_SORT_BINS - 2);
}

__global__ void k_sort_count(DevScene S, PathSoA P, uint32_t depth) {
    const uint32_t n = P.ctl->count[depth];
    const int lane = threadIdx.x & 31;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t key = shade_key(S, P.hit_inst[j]);
        const unsigned peers = __match_any_sync(__activemask(), key);
        if (lane == __ffs(peers) - 1) atomicAdd(&P.ctl->sort_hist[key], (uint32_t)__popc(peers));
    }
}

// One block of PYRE_SORT_BINS threads: exclusive scan of the bin sizes into
// the bin offsets; the sizes are cleared for the next sort.
__global__ void __launch_bounds__(PYRE_SORT_BINS) k_sort_scan(PathSoA P) {
    __shared__ uint32_t warp_sum[PYRE_SORT_BINS / 32];
    const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t v = P.ctl->sort_hist[t];
    P.ctl->sort_hist[t] = 0;
    uint32_t x = v;  // inclusive scan within the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        warp_sum[lane] = w;  // inclusive sums of the warps
    }
    __syncthreads();
    P.ctl->sort_off[t] = (warp ? warp_sum[warp - 1] : 0u) + x - v;
}

__global__ void k_sort_scatter(DevScene S, PathSoA P, uint32_t depth) {
    const uint32_t n = P.ctl->count[depth];
    const int lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t key = shade_key(S, P.hit_inst[j]);
        const unsigned peers = __match_any_sync(__activemask(), key);
        const int leader = __ffs(peers) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&P.ctl->sort_off[key], (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        P.qsort[base + __popc(peers & below)] = j;  // the queue position
    }
}

// Material sort within tiles of PYRE_SORT_TILE_N consecutive queue entries:
// one block sorts a tile by shade key in shared memory (a warp-aggregated
// histogram, a block scan, a scatter) and writes the tile's part of P.qsort.
// Shade's warps mostly see one material at a time, while its path-state reads
// stay within the tile. On the 1080p studio frame (65 materials, Disney BSDFs,
// environment NEE), with tiles of 2048 entries: 781.2 against 770.9
// Msamples/s unsorted (shade 41.5 against 43.3 ms, and the next extend 91.7
// against 92.0); sorting the whole queue gave 733.6. On the Cornell views of the batch workload (Lambertian
// walls, quad-light NEE) shade is bound by its path-state traffic, and the
// sorted order, which spreads a warp's path indices over the tile, doubles
// its time at bounces 1-3 (9.3 against 5.0 ms at bounce 1 of a 1024^2 view at
// 64 spp). Rendering therefore leaves the queue unsorted unless asked.
// Within a tile, paths of one key land in any order; shade's results do not
// depend on the order in which it visits paths.
// Queue entries per tile, PYRE_SORT_TILE_E per thread of a 256-thread block:
// on the 1080p studio frame 1024 / 2048 / 4096 / 8192 / 16384 entries gave
// 766.5 / 784.2 / 793.4 / 791.0 / 782.4 Msamples/s.
#ifndef PYRE_SORT_TILE_N
#define PYRE_SORT_TILE_N 4096
#endif
#define PYRE_SORT_TILE_E (PYRE_SORT_TILE_N / 256)
static_assert(PYRE_SORT_TILE_N % 256 == 0 && PYRE_SORT_TILE_N >= 256, "a tile is whole 256-thread rows");
static_assert(PYRE_SORT_BINS % 256 == 0, "k_sort_tile scans PYRE_SORT_BINS / 256 bins per thread");
__global__ void __launch_bounds__(256) k_sort_tile(DevScene S, PathSoA P, uint32_t depth) {
    __shared__ uint32_t hist[PYRE_SORT_BINS];
    __shared__ uint32_t wsum[8];
    const uint32_t n = P.ctl->count[depth];
    const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const unsigned below = (1u << lane) - 1u;
    for (uint32_t base = blockIdx.x * PYRE_SORT_TILE_N; base < n; base += gridDim.x * PYRE_SORT_TILE_N) {
        for (uint32_t k = t; k < PYRE_SORT_BINS; k += 256) hist[k] = 0;
        __syncthreads();
        uint32_t key[PYRE_SORT_TILE_E], rank[PYRE_SORT_TILE_E];
#pragma unroll
        for (int e = 0; e < PYRE_SORT_TILE_E; ++e) {
            const uint32_t j = base + e * 256 + t;
            key[e] = j < n ? shade_key(S, __ldcs(P.hit_inst + j)) : PYRE_SORT_BINS;
            const unsigned peers = __match_any_sync(0xffffffffu, key[e]);
            const int leader = __ffs(peers) - 1;
            uint32_t b = 0;
            if (key[e] < PYRE_SORT_BINS && (int)lane == leader) b = atomicAdd(&hist[key[e]], (uint32_t)__popc(peers));
            rank[e] = __shfl_sync(0xffffffffu, b, leader) + __popc(peers & below);
        }
        __syncthreads();
        // exclusive scan of the bins: 4 per thread, then across the block
        uint32_t v[PYRE_SORT_BINS / 256], sum = 0;
#pragma unroll
        for (int q = 0; q < PYRE_SORT_BINS / 256; ++q) { v[q] = hist[(PYRE_SORT_BINS / 256) * t + q]; sum += v[q]; }
        uint32_t x = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= (uint32_t)o) x += y;
        }
        if (lane == 31) wsum[warp] = x;
        __syncthreads();
        uint32_t off = x - sum;
        for (uint32_t w = 0; w < warp; ++w) off += wsum[w];
#pragma unroll
        for (int q = 0; q < PYRE_SORT_BINS / 256; ++q) { hist[(PYRE_SORT_BINS / 256) * t + q] = off; off += v[q]; }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < PYRE_SORT_TILE_E; ++e) {
            const uint32_t j = base + e * 256 + t;
            if (j < n) P.qsort[base + hist[key[e]] + rank[e]] = j;
        }
        __syncthreads();
    }
}

// ----------------------------------------------------------------- shade --
// One path vertex of PathIntegrator::integrate (integrator.rs:242-388).
// ADJ: the path-replay adjoint of the same vertex (pyre_backward): the same
// draws and decisions, plus the derivatives of its terms.
// Forward shade: 4 resident blocks of 224 threads (72 registers); it is
// latency-bound, and 28 warps per SM beat 24 (3 blocks of 256, 80
// registers) by 0.3 % on the 1080p studio frame. The adjoint variant keeps
// 3 blocks of 256: at 72 registers its spills would grow.
template <bool BATCH, bool ADJ = false>
__global__ void __launch_bounds__(ADJ ? 256 : PYRE_SHADE_THREADS, ADJ ? 3 : PYRE_SHADE_BLOCKS) k_shade(DevScene S, PathSoA P, WaveParams W,
                                                                        uint32_t depth) {
    GradSmem G{nullptr, nullptr, nullptr};
    if (ADJ) G = grad_smem_begin(W.env_cache != 0, W.smem_grad != 0, W.n_mat);
    const uint32_t n = P.ctl->count[depth];
    const uint32_t* qin = P.q[depth & 1];
    uint32_t* qout = P.q[(depth + 1) & 1];
    uint32_t* next_count = &P.ctl->count[depth + 1];
    uint32_t* shadow_count = &P.ctl->scount[depth];
    const bool last_was_specular = depth == 0;  // no specular BSDFs: only camera rays
    const float INF = __int_as_float(0x7f800000);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        // queue position of the path's ray and hit (depth 0: the path index), and the path
        const uint32_t pos = W.sort ? P.qsort[j] : (depth > 0 ? j : (BATCH ? j : tiled_path(W, j)));
        const uint32_t i = depth > 0 ? __ldcs(qin + pos) : pos;
        // a batch ray carries its job in the origin's w
        float4 ro_b = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (BATCH) ro_b = __ldcs(P.ray_o[depth & 1] + pos);
        const DevJob* JB = BATCH ? &W.jobs[__float_as_uint(ro_b.w)] : nullptr;
        // a batch wave traces every job's camera rays; a job with max_depth 0 shades none
        if (BATCH && depth == 0 && JB->max_depth == 0) continue;
        // a camera path starts with radiance 0 and throughput 1 (integrator.rs:63-64)
        float4 Lq = make_float4(0.0f, 0.0f, 0.0f, 0.0f), bq = make_float4(1.0f, 1.0f, 1.0f, 0.0f);
        if (depth > 0) ldcs_256(P.Lb + 2 * (size_t)i, Lq, bq);
        f3 L = mk3(Lq.x, Lq.y, Lq.z);
        f3 delta = splat3(0.0f), Ltot = splat3(0.0f);
        if (ADJ) {  // adjoint of this path's film pixel, and its forward radiance
            const uint32_t k = i / W.npix, pp = i - k * W.npix;
            delta = mk3(W.dl_di[3 * (size_t)pp], W.dl_di[3 * (size_t)pp + 1], W.dl_di[3 * (size_t)pp + 2]) * W.inv_spp;
            const float4 lt = P.keep_L[(size_t)(P.ctl->s_base - W.spp_begin + k) * W.npix + pp];
            Ltot = mk3(lt.x, lt.y, lt.z);
        }
        // Contributions left by the previous vertex's NEE, in light order.
        GradTerms gt;  // ADJ: this vertex's terms for the previous vertex's material
        if (depth > 0) {
            for (uint32_t s = 0; s < W.ns; ++s) {
                float4 c = __ldcs(P.pend + (size_t)i * W.ns + s);
                if (c.w != 0.0f) {
                    L = L + mk3(c.x, c.y, c.z);
                    __stcs(&P.pend[(size_t)i * W.ns + s], make_float4(0.0f, 0.0f, 0.0f, 0.0f));
                    if (ADJ) collect_parked_grad(P.gpend + PYRE_GSLOT * ((size_t)i * W.ns + s), gt);
                }
            }
            if (ADJ) {
                // BSDF sample of the previous vertex: beta_d * a * R_{d+1} = (L_total - L_so_far) / f
                const float4 b0 = P.brec[3 * (size_t)i], b1 = P.brec[3 * (size_t)i + 1], b2 = P.brec[3 * (size_t)i + 2];
                if (b1.w != 0.0f) {
                    const f3 after = Ltot - L;
                    const f3 w = mk3(b2.x > 0.0f ? delta.x * after.x / b2.x : 0.0f,
                                     b2.y > 0.0f ? delta.y * after.y / b2.y : 0.0f,
                                     b2.z > 0.0f ? delta.z * after.z / b2.z : 0.0f);
                    if (!is_zero3(w)) {
                        const uint32_t m = __float_as_uint(b0.w);
                        float g[6];
                        jac_dot(load_bsdf(S, m), mk3(b0.x, b0.y, b0.z), mk3(b1.x, b1.y, b1.z), w, g);
                        gt.mat = m;
#pragma unroll
                        for (int k = 0; k < PYRE_NPARAM; ++k) gt.g[k] += g[k];
                    }
                }
            }
        }
        if (ADJ) warp_flush(S, W.env_grad, W.mat_grad, G, gt);
        f3 beta = mk3(bq.x, bq.y, bq.z);
        const float last_pdf = bq.w;
        float next_pdf = last_pdf;  // stored with the throughput: the pdf of this vertex's BSDF sample
        const float4 ro = BATCH ? ro_b : __ldcs(P.ray_o[depth & 1] + pos), rd = __ldcs(P.ray_d[depth & 1] + pos);
        const f3 ray_o = mk3(ro.x, ro.y, ro.z), ray_d = mk3(rd.x, rd.y, rd.z);
        const float time = rd.w;
        const float4 hq = __ldcs(P.hit + pos);
        const int32_t code = __ldcs(P.hit_inst + pos);

        if (code == -1) {
            if (depth == 0) {  // a camera ray that escapes leaves the AOVs at zero
                stcs_256(P.aov + 2 * (size_t)i, make_float4(0.0f, 0.0f, 0.0f, 0.0f),
                         make_float4(0.0f, 0.0f, 0.0f, 0.0f));
            }
            // Escaped: environment radiance with MIS against the BSDF arm (integrator.rs:243-259).
            if (S.has_env) {
                const f2 uv = env_dir_to_uv(ray_d);
                f3 le = env_texture(S.env, uv) * S.env.intensity;
                if (!is_zero3(le)) {
                    float w_adj = 1.0f;
                    if (last_was_specular) L = L + beta * le;
                    else {
                        float pdf_env = env_pdf_at(S.env, uv);
                        float w = power_heuristic(last_pdf, pdf_env);
                        L = L + beta * le * w;
                        w_adj = w;
                    }
                    // d/d texels of beta * texture(uv) * intensity * w
                    if (ADJ) scatter_env(S.env, W.env_grad, G, uv, delta * beta * w_adj);
                }
            }
        } else if (code <= -2) {
            // Quad light hit (integrator.rs:262-295).
            const DevQuadLight& Lt = S.lights[-2 - code];
            if (depth == 0) {
                stcs_256(P.aov + 2 * (size_t)i, make_float4(1.0f, 1.0f, 1.0f, hq.x),
                         make_float4(Lt.normal.x, Lt.normal.y, Lt.normal.z, 0.0f));
            }
            f3 le = dot3(Lt.normal, -ray_d) > 0.0f ? Lt.emission : splat3(0.0f);
            if (last_was_specular) L = L + beta * le;
            else {
                float pdf_light = quad_pdf(Lt, ray_o, ray_d);
                float w = power_heuristic(last_pdf, pdf_light);
                L = L + beta * le * w;
            }
        } else {
            // Surface hit: position and shading normal (mesh.rs:126-136,147).
            const DevInstance& I = S.inst[code];
            const float t = hq.x, u = hq.y, v = hq.z;
            const int32_t slot = __float_as_int(hq.w);
            f3 off = splat3(0.0f);
            if (I.has_motion) off = motion_offset(I, time);
            const bool moved = !is_zero3(off);
            f3 o_local = moved ? ray_o - off : ray_o;
            f3 p = o_local + ray_d * t;
            if (moved) p = p + off;
            f3 ns;
            // the slot's vertex normals: one record, does not wait for the instance
            const float4 n0 = __ldg(S.slot_normals + 3 * (size_t)slot), n1 = __ldg(S.slot_normals + 3 * (size_t)slot + 1),
                         n2 = __ldg(S.slot_normals + 3 * (size_t)slot + 2);
            if (I.normal_base >= 0) {
                const f3 na = mk3(n0.x, n0.y, n0.z), nb = mk3(n1.x, n1.y, n1.z), nc = mk3(n2.x, n2.y, n2.z);
                const float w = 1.0f - u - v;
                ns = normalize3(w * na + u * nb + v * nc);
            } else {
                const float4 B = __ldg(S.tris + 3 * (size_t)slot + 1), C = __ldg(S.tris + 3 * (size_t)slot + 2);
                ns = normalize3(cross3(mk3(B.x, B.y, B.z), mk3(C.x, C.y, C.z)));
            }
            const Bsdf mat = load_bsdf(S, I.material);
            if (depth == 0) {
                stcs_256(P.aov + 2 * (size_t)i, make_float4(mat.base.x, mat.base.y, mat.base.z, t),
                         make_float4(ns.x, ns.y, ns.z, 0.0f));
            }
            const Frame3 fr = frame_from_normal(ns);
            const f3 wo = to_local(fr, -ray_d);
            if (wo.z > 0.0f) {
                Rng g = load_rng(P.rng, i);
                const f3 p_off = p + 1e-3f * ns;
                uint32_t lfirst = 0, lcount = S.n_lights;
                if (BATCH) {
                    lfirst = JB->light_first; lcount = JB->light_count;
                }
                // The vertex's sampling arms in the reference's order, each
                // drawing its two numbers first: NEE for every quad light
                // (integrator.rs:307-333), NEE for the environment (335-354),
                // then the BSDF sample (356-387). All three evaluate the BSDF
                // at one call site, so the kernel holds one copy of it.
                const uint32_t n_nee = lcount + (S.has_env ? 1u : 0u);
                for (uint32_t s = 0; s <= n_nee; ++s) {
                    const f2 u2 = g.next_vec2();
                    const bool bsdf_arm = s == n_nee, env_arm = !bsdf_arm && s == lcount;
                    f3 wi, wi_w = splat3(0.0f), le = splat3(0.0f), sh_dir = splat3(0.0f);
                    float lpdf = 0.0f, sh_tmax = INF;
                    bool sh_ray = true;
                    if (bsdf_arm) {
                        if (!bsdf_sample_dir(mat, wo, u2, &wi)) break;
                    } else if (!env_arm) {
                        const DevQuadLight& Lt = S.lights[lfirst + s];
                        f3 lpos;
                        if (!quad_sample(Lt, p, u2, &lpos, &wi_w, &lpdf)) continue;
                        if (lpdf <= 0.0f || is_zero3(Lt.emission)) continue;
                        wi = to_local(fr, wi_w);
                        if (wi.z <= 0.0f) continue;
                        le = Lt.emission;
                        // Scene::occluded (scene.rs:120-140) towards the light point
                        const f3 tf = (lpos - 1e-3f * wi_w) - p_off;
                        const float dist = len3(tf);
                        sh_ray = dist > 0.0f;
                        sh_dir = tf / dist;
                        sh_tmax = dist - 1e-3f;
                    } else {
                        env_sample(S.env, u2, W.env_cdf, &wi_w, &le, &lpdf);
                        if (!(lpdf > 0.0f) || is_zero3(le)) continue;
                        wi = to_local(fr, wi_w);
                        if (wi.z <= 0.0f) continue;
                        sh_dir = wi_w;
                    }
                    f3 f;
                    float pdf_b;
                    bsdf_eval_pdf(mat, wo, wi, &f, &pdf_b);
                    if (bsdf_arm) {
                        // Bsdf::sample is None for a non-positive Disney pdf;
                        // the integrator also needs pdf > 0 and cos != 0.
                        if (!(pdf_b > 0.0f)) break;
                        const float cos_wi = fabsf(wi.z);
                        if (cos_wi == 0.0f) break;
                        beta = beta * (f * cos_wi / pdf_b);
                        bool survive = true;
                        if (depth >= (BATCH ? JB->min_rr : W.min_rr)) {
                            float q = clampf_(1.0f - max_elem3(beta), 0.05f, 0.95f);
                            if (g.next_f32() < q) survive = false;
                            else beta = beta / (1.0f - q);
                        }
                        if (survive) {
                            // Next ray (integrator.rs:377-387), at the path's
                            // position in the next depth's queue
                            if (depth + 1 < (BATCH ? JB->max_depth : W.max_depth)) {
                                const f3 nd = to_world(fr, wi);
                                const uint32_t q = append_slot(next_count);
                                qout[q] = i;
                                __stcs(P.ray_o[(depth + 1) & 1] + q,
                                       make_float4(p_off.x, p_off.y, p_off.z, BATCH ? ro.w : 1e-4f));
                                __stcs(P.ray_d[(depth + 1) & 1] + q, make_float4(nd.x, nd.y, nd.z, time));
                            }
                            next_pdf = pdf_b;
                            if (ADJ) {  // for the next vertex's BSDF-sample gradient
                                P.brec[3 * (size_t)i] = make_float4(wo.x, wo.y, wo.z, __uint_as_float(I.material));
                                P.brec[3 * (size_t)i + 1] = make_float4(wi.x, wi.y, wi.z, 1.0f);
                                P.brec[3 * (size_t)i + 2] = make_float4(f.x, f.y, f.z, 0.0f);
                            }
                        }
                        break;
                    }
                    if (is_zero3(f)) continue;
                    const float w = power_heuristic(lpdf, pdf_b);
                    const f3 contrib = beta * f * le * wi.z * w / lpdf;
                    const size_t sidx = (size_t)i * W.ns + (env_arm ? S.n_lights : s);
                    __stcs(&P.pend[sidx], make_float4(contrib.x, contrib.y, contrib.z, 1.0f));
                    if (ADJ) {  // park the slot's d/d params (and texels); cleared if occluded
                        float4* G = P.gpend + PYRE_GSLOT * sidx;
                        float gm[6];
                        // quad light: beta * f * (Le cos w / pdf); environment:
                        // beta * f * (texture * intensity) * k, k = cos w / pdf.
                        // One Jacobian call site for both arms keeps the kernel's
                        // code (and its instruction-cache misses) smaller.
                        const float k = wi.z * w / lpdf;
                        jac_dot(mat, wo, wi, delta * beta * (env_arm ? le * k : le * wi.z * w / lpdf), gm);
                        if (!env_arm) {
                            G[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        } else {
                            const f2 uv = env_dir_to_uv(wi_w);
                            const f3 ke = delta * beta * f * k;
                            G[2] = make_float4(uv.x, uv.y, 1.0f, 0.0f);
                            G[3] = make_float4(ke.x, ke.y, ke.z, 0.0f);
                        }
                        G[0] = make_float4(gm[0], gm[1], gm[2], gm[3]);
                        G[1] = make_float4(gm[4], gm[5], __uint_as_float(I.material), 1.0f);
                    }
                    if (sh_ray) {
                        const uint32_t q = append_slot(shadow_count);
                        __stcs(P.sh_o + q, make_float4(p_off.x, p_off.y, p_off.z, sh_tmax));
                        __stcs(P.sh_d + q, make_float4(sh_dir.x, sh_dir.y, sh_dir.z, time));
                        P.sq[q] = (uint32_t)sidx;
                        if (BATCH) __stcs(P.sroot + q, JB->tlas_root);
                    }
                }
                store_rng(P.rng, i, g);
            }
        }
        // a path without a next ray is not read again, whatever its throughput
        stcs_256(P.Lb + 2 * (size_t)i, make_float4(L.x, L.y, L.z, 0.0f), make_float4(beta.x, beta.y, beta.z, next_pdf));
    }
    if (ADJ) grad_smem_end(G, W.env_grad, W.mat_grad, W.n_mat);  // one atomic per parameter / texel per block
}

// Adjoint replay: parked gradient terms of the paths' last vertices.
__global__ void k_accumulate_adjoint(DevScene S, PathSoA P, WaveParams W) {
    const GradSmem G = grad_smem_begin(W.env_cache != 0, W.smem_grad != 0, W.n_mat);
    const uint32_t n = P.ctl->n_valid;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        GradTerms gt;
        for (uint32_t s = 0; s < W.ns; ++s)
            if (P.pend[(size_t)i * W.ns + s].w != 0.0f)
                collect_parked_grad(P.gpend + PYRE_GSLOT * ((size_t)i * W.ns + s), gt);
        warp_flush(S, W.env_grad, W.mat_grad, G, gt);
    }
    grad_smem_end(G, W.env_grad, W.mat_grad, W.n_mat);
}

// ------------------------------------------------------------ accumulate --
// Film sums in sample order (main.rs:275-278): pending NEE of the last vertex
// is added to the path radiance first.
__global__ void k_accumulate(PathSoA P, WaveParams W) {
    const uint32_t kv = P.ctl->k_valid;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < W.npix; p += gridDim.x * blockDim.x) {
        float4 ar = P.acc_r[p], aa = P.acc_a[p], an = P.acc_n[p];
        f3 mean = splat3(0.0f);
        if (W.prog_mean && P.ctl->s_base > 0)
            mean = mk3(W.prog_mean[3 * (size_t)p], W.prog_mean[3 * (size_t)p + 1], W.prog_mean[3 * (size_t)p + 2]);
        for (uint32_t k = 0; k < kv; ++k) {
            uint32_t i = k * W.npix + p;
            const float4 Lq = __ldcs(P.Lb + 2 * (size_t)i);  // last reads of the path state
            f3 L = mk3(Lq.x, Lq.y, Lq.z);
            for (uint32_t s = 0; s < W.ns; ++s) {
                const float4 c = __ldcs(P.pend + (size_t)i * W.ns + s);
                if (c.w != 0.0f) L = L + mk3(c.x, c.y, c.z);
            }
            if (W.prog_mean) {
                // the viewer's merge of pass s (viewer.rs:164-177): mean += (L - mean) / (s + 1)
                const float n = (float)(P.ctl->s_base + k + 1);
                mean = mean + (L - mean) / n;
            }
            float4 a, nn;
            ldcs_256(P.aov + 2 * (size_t)i, a, nn);
            ar.x += L.x; ar.y += L.y; ar.z += L.z; ar.w += a.w;
            aa.x += a.x; aa.y += a.y; aa.z += a.z;
            an.x += nn.x; an.y += nn.y; an.z += nn.z;
            if (P.keep_L)  // pyre_forward: the path's radiance, for the adjoint replay
                P.keep_L[(size_t)(P.ctl->s_base - W.spp_begin + k) * W.npix + p] = make_float4(L.x, L.y, L.z, 0.0f);
        }
        P.acc_r[p] = ar; P.acc_a[p] = aa; P.acc_n[p] = an;
        if (W.prog_mean) {
            W.prog_mean[3 * (size_t)p] = mean.x;
            W.prog_mean[3 * (size_t)p + 1] = mean.y;
            W.prog_mean[3 * (size_t)p + 2] = mean.z;
        }
    }
}

// Batch: one thread per (segment, pixel) slot of the wave; samples of the
// segment are added in sample order into the job's accumulators.
__global__ void k_accumulate_batch(PathSoA P, WaveParams W) {
    const DevWave wv = W.waves[P.ctl->wave];
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < wv.n_slots; q += gridDim.x * blockDim.x) {
        const DevSeg sg = W.segs[find_segment(W.segs, wv, q, true)];
        const DevJob& J = W.jobs[sg.job];
        const uint32_t p = q - sg.slot_base;
        const uint32_t a = J.acc_base + p;
        float4 ar = P.acc_r[a], aa = P.acc_a[a], an = P.acc_n[a];
        for (uint32_t k = 0; k < sg.s_count; ++k) {
            const uint32_t i = sg.path_base + k * J.npix + p;
            const float4 Lq = __ldcs(P.Lb + 2 * (size_t)i);  // last reads of the path state
            f3 L = mk3(Lq.x, Lq.y, Lq.z);
            for (uint32_t s = 0; s < W.ns; ++s) {
                const float4 c = __ldcs(P.pend + (size_t)i * W.ns + s);
                if (c.w != 0.0f) L = L + mk3(c.x, c.y, c.z);
            }
            float4 al, nn;
            ldcs_256(P.aov + 2 * (size_t)i, al, nn);
            ar.x += L.x; ar.y += L.y; ar.z += L.z; ar.w += al.w;
            aa.x += al.x; aa.y += al.y; aa.z += al.z;
            an.x += nn.x; an.y += nn.y; an.z += nn.z;
        }
        P.acc_r[a] = ar; P.acc_a[a] = aa; P.acc_n[a] = an;
    }
}

// Batch: per-job means into a staging film laid out like the accumulators.
// Means of the batch accumulators [a0, a1) (whole jobs) into the staging film.
__global__ void k_finalize_batch(PathSoA P, const DevJob* jobs, uint32_t n_jobs, uint32_t total, uint32_t a0,
                                 uint32_t a1, float* out) {
    for (uint32_t a = a0 + blockIdx.x * blockDim.x + threadIdx.x; a < a1; a += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n_jobs - 1;
        while (lo < hi) {
            uint32_t mid = (lo + hi + 1) / 2;
            if (jobs[mid].acc_base <= a) lo = mid; else hi = mid - 1;
        }
        const float inv = jobs[lo].inv_spp;
        float4 ar = P.acc_r[a], aa = P.acc_a[a], an = P.acc_n[a];
        float* rad = out;
        float* alb = out + 3 * (size_t)total;
        float* nor = out + 6 * (size_t)total;
        float* dep = out + 9 * (size_t)total;
        rad[3 * (size_t)a] = ar.x * inv; rad[3 * (size_t)a + 1] = ar.y * inv; rad[3 * (size_t)a + 2] = ar.z * inv;
        alb[3 * (size_t)a] = aa.x * inv; alb[3 * (size_t)a + 1] = aa.y * inv; alb[3 * (size_t)a + 2] = aa.z * inv;
        nor[3 * (size_t)a] = an.x * inv; nor[3 * (size_t)a + 1] = an.y * inv; nor[3 * (size_t)a + 2] = an.z * inv;
        dep[a] = ar.w * inv;
    }
}

// Mean over the sample range (main.rs:280-285).
__global__ void k_finalize(PathSoA P, uint32_t npix, float inv_spp, float* rad, float* alb, float* nor, float* dep) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        float4 ar = P.acc_r[p], aa = P.acc_a[p], an = P.acc_n[p];
        if (rad) { rad[3 * (size_t)p] = ar.x * inv_spp; rad[3 * (size_t)p + 1] = ar.y * inv_spp; rad[3 * (size_t)p + 2] = ar.z * inv_spp; }
        if (alb) { alb[3 * (size_t)p] = aa.x * inv_spp; alb[3 * (size_t)p + 1] = aa.y * inv_spp; alb[3 * (size_t)p + 2] = aa.z * inv_spp; }
        if (nor) { nor[3 * (size_t)p] = an.x * inv_spp; nor[3 * (size_t)p + 1] = an.y * inv_spp; nor[3 * (size_t)p + 2] = an.z * inv_spp; }
        if (dep) dep[p] = ar.w * inv_spp;
    }
}

// ------------------------------------------------------ ray-query kernels --
// Rays and results of pyre_intersect_closest / pyre_intersect_any (caller
// arrays, SoA).
struct QueryRays {
    static constexpr float kTmin = 0.0f, kTmax = 0.0f;  // both come with each ray
    const DevScene* S;
    const float* org; const float* dir; const float* tmin; const float* tmax; const float* time;
    int32_t* kind; int32_t* inst; int32_t* tri; float* tt; float* uu; float* vv; uint8_t* occluded;
    __device__ __forceinline__ uint32_t load(uint32_t i, TraceRay& r, int32_t& root) const {
        r.o = mk3(org[3 * (size_t)i], org[3 * (size_t)i + 1], org[3 * (size_t)i + 2]);
        r.d = mk3(dir[3 * (size_t)i], dir[3 * (size_t)i + 1], dir[3 * (size_t)i + 2]);
        r.tmin = tmin[i];
        r.tmax = tmax[i];
        r.time = time ? time[i] : 0.0f;
        root = S->tlas_root;
        return i;
    }
    __device__ __forceinline__ void store(uint32_t i, const TraceRay& r, TraceHit& h, bool found) const {
        if (occluded) { occluded[i] = found ? 1 : 0; return; }
        hit_quad_lights(*S, r, 0, S->n_lights, &h);
        if (h.light >= 0) {
            kind[i] = 2; inst[i] = h.light; tri[i] = -1;
            tt[i] = h.t; uu[i] = 0.0f; vv[i] = 0.0f;
        } else if (h.inst >= 0) {
            kind[i] = 1;
            inst[i] = S->inst[h.inst].orig_id;
            tri[i] = (int32_t)__float_as_uint(__ldg(S->tris + 3 * (size_t)h.tri).w);
            tt[i] = h.t; uu[i] = h.u; vv[i] = h.v;
        } else {
            kind[i] = 0; inst[i] = -1; tri[i] = -1;
            tt[i] = __int_as_float(0x7f800000); uu[i] = 0.0f; vv[i] = 0.0f;
        }
    }
};

template <bool ANY, int WIDTH>
__global__ void __launch_bounds__(128, ANY ? PYRE_TRACE_BLOCKS_ANY : PYRE_TRACE_BLOCKS) k_intersect(DevScene S, QueryRays q, uint32_t n, unsigned int* counter,
                                                   int refill) {
    QueryRays src = q;
    src.S = &S;
    trace_stream<ANY, WIDTH>(S, src, n, counter, refill);
}

// ------------------------------------------------------------ host side --
namespace {

template <typename K>
int grid_for(pyre_ctx* ctx, K kernel, int block, size_t smem = 0) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
    return std::max(1, per_sm) * std::max(1, ctx->num_sms);
}

// Carves the workspace into typed arrays (256-byte aligned).
struct Carver {
    char* base;
    size_t off = 0;
    template <typename T>
    T* take(size_t count) {
        off = (off + 255) & ~(size_t)255;
        T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
        off += count * sizeof(T);
        return p;
    }
};

size_t carve_paths(char* base, size_t P, uint32_t ns, uint32_t npix, PathSoA* out, bool batch = false,
                   bool adjoint = false) {
    Carver c{base};
    PathSoA s;
    s.ray_o[0] = c.take<float4>(P);
    s.ray_o[1] = c.take<float4>(P);
    s.ray_d[0] = c.take<float4>(P);
    s.ray_d[1] = c.take<float4>(P);
    s.hit = c.take<float4>(P);
    s.hit_inst = c.take<int32_t>(P);
    s.rng = c.take<uint4>(2 * P);
    s.Lb = c.take<float4>(2 * P);
    s.aov = c.take<float4>(2 * P);
    s.pend = c.take<float4>(P * ns);
    s.sh_o = c.take<float4>(P * ns);
    s.sh_d = c.take<float4>(P * ns);
    s.q[0] = c.take<uint32_t>(P);
    s.q[1] = c.take<uint32_t>(P);
    s.qsort = c.take<uint32_t>(P);
    s.sq = c.take<uint32_t>(P * ns);
    s.acc_r = c.take<float4>(npix);
    s.acc_a = c.take<float4>(npix);
    s.acc_n = c.take<float4>(npix);
    s.ctl = c.take<WaveCtl>(1);
    s.sroot = batch ? c.take<int32_t>(P * ns) : nullptr;
    s.keep_L = nullptr;
    s.gpend = adjoint ? c.take<float4>(P * ns * PYRE_GSLOT) : nullptr;
    s.brec = adjoint ? c.take<float4>(3 * P) : nullptr;
    if (out) *out = s;
    return c.off + 256;
}

// Default wave capacity: the paths whose state fits a quarter of the device
// memory that is free (counting this context's own path workspace), between
// 8 Mi and 128 Mi paths. On the 1080p 64-spp studio frame 8, 16, 32, 64 and
// 128 Mi paths gave 444, 479, 497, 506 and 510 Msamples/s: the last bounces
// of a wave hold few live paths, and a larger wave spends a smaller share of
// those launches draining the warps' final rays.
uint64_t default_wave_paths(pyre_ctx* ctx, uint32_t ns, bool batch, bool adjoint) {
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        cudaGetLastError();
        return (uint64_t)8 << 20;
    }
    const uint64_t per_path =
        std::max<uint64_t>(1, carve_paths(nullptr, (size_t)1 << 20, std::max(ns, 1u), 0, nullptr, batch, adjoint) >> 20);
    const uint64_t n = ((uint64_t)free_b + ctx->render_ws.bytes) / 4 / per_path;
    return std::min<uint64_t>(std::max<uint64_t>(n, (uint64_t)8 << 20), (uint64_t)128 << 20);
}

struct Launch {
    int block_stage = 256;  // raygen, accumulate, adjoint shade (at most 256)
    int block_shade = PYRE_SHADE_THREADS;  // forward shade (at most PYRE_SHADE_THREADS)
    int block_trace = 128;  // extend, shadow (at most 128)
    int grid_raygen, grid_shade, grid_extend, grid_shadow, grid_acc, grid_sort;
};

// Grid sizes for the stage kernels: persistent grids of resident blocks.
// block_size (0 = defaults: 256 for raygen and accumulate, 224 for the
// forward shade, 128 for the traces) sets them all, capped at 224 for the
// forward shade and 128 for the traces.
template <bool BATCH>
Launch make_launch(pyre_ctx* ctx, uint32_t block_size, int width) {
    Launch L;
    if (block_size) {
        const int b = (int)std::max(32u, std::min(256u, block_size / 32 * 32));
        L.block_stage = b;
        L.block_shade = std::min(b, PYRE_SHADE_THREADS);
        L.block_trace = std::min(b, 128);
    }
    L.grid_raygen = grid_for(ctx, k_raygen<BATCH>, L.block_stage);
    L.grid_shade = grid_for(ctx, k_shade<BATCH>, L.block_shade);
    L.grid_extend = width == 8 ? grid_for(ctx, k_extend<BATCH, 8>, L.block_trace)
                    : width == 4 ? grid_for(ctx, k_extend<BATCH, 4>, L.block_trace)
                                 : grid_for(ctx, k_extend<BATCH, 2>, L.block_trace);
    L.grid_shadow = width == 8 ? grid_for(ctx, k_shadow<BATCH, 8>, L.block_trace)
                    : width == 4 ? grid_for(ctx, k_shadow<BATCH, 4>, L.block_trace)
                                 : grid_for(ctx, k_shadow<BATCH, 2>, L.block_trace);
    L.grid_acc = BATCH ? grid_for(ctx, k_accumulate_batch, L.block_stage) : grid_for(ctx, k_accumulate, L.block_stage);
    L.grid_sort = grid_for(ctx, k_sort_scatter, 256);
    return L;
}

// Stage timing (off by default): an event before each stage kernel, tagged
// with that kernel's stage; durations are differences of consecutive events.
void mark(pyre_ctx* ctx, int tag) {
    if (!ctx->stage_timing) return;
    if (ctx->stage_used == ctx->stage_ev.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        ctx->stage_ev.push_back(e);
        ctx->stage_tag.push_back(0);
    }
    ctx->stage_tag[ctx->stage_used] = tag;
    cudaEventRecord(ctx->stage_ev[ctx->stage_used++], ctx->stream);
}

enum { STAGE_EXTEND = 0, STAGE_SHADE = 1, STAGE_SHADOW = 2, STAGE_OTHER = 3, STAGE_END = 4 };

// The traversal kernels for the render's BVH width.
template <bool BATCH>
void launch_extend(cudaStream_t st, const Launch& Lc, const DevScene& S, const PathSoA& P, const WaveParams& W,
                   uint32_t d) {
    if (W.bvh_width == 8) k_extend<BATCH, 8><<<Lc.grid_extend, Lc.block_trace, 0, st>>>(S, P, W, d);
    else if (W.bvh_width == 4) k_extend<BATCH, 4><<<Lc.grid_extend, Lc.block_trace, 0, st>>>(S, P, W, d);
    else k_extend<BATCH, 2><<<Lc.grid_extend, Lc.block_trace, 0, st>>>(S, P, W, d);
}
template <bool BATCH>
void launch_shadow(cudaStream_t st, const Launch& Lc, const DevScene& S, const PathSoA& P, const WaveParams& W,
                   uint32_t d) {
    if (W.bvh_width == 8) k_shadow<BATCH, 8><<<Lc.grid_shadow, Lc.block_trace, 0, st>>>(S, P, W, d);
    else if (W.bvh_width == 4) k_shadow<BATCH, 4><<<Lc.grid_shadow, Lc.block_trace, 0, st>>>(S, P, W, d);
    else k_shadow<BATCH, 2><<<Lc.grid_shadow, Lc.block_trace, 0, st>>>(S, P, W, d);
}

// Orders the live paths of depth d by shade_key into P.qsort.
// W.sort: PYRE_SORT_TILES sorts within tiles of the queue (one launch),
// PYRE_SORT_QUEUE the whole queue (three launches).
void enqueue_sort(pyre_ctx* ctx, const DevScene& S, const PathSoA& P, const Launch& Lc, uint32_t d, int kind) {
    cudaStream_t st = ctx->stream;
    if (kind == PYRE_SORT_TILES) {
        k_sort_tile<<<Lc.grid_sort, 256, 0, st>>>(S, P, d);
        return;
    }
    k_sort_count<<<Lc.grid_sort, 256, 0, st>>>(S, P, d);
    k_sort_scan<<<1, PYRE_SORT_BINS, 0, st>>>(P);
    k_sort_scatter<<<Lc.grid_sort, 256, 0, st>>>(S, P, d);
}

void enqueue_wave(pyre_ctx* ctx, const DevScene& S, const PathSoA& P, const WaveParams& W, const Launch& Lc) {
    cudaStream_t st = ctx->stream;
    mark(ctx, STAGE_OTHER);
    k_wave_begin<<<1, 32, 0, st>>>(P.ctl, W.spp_begin, W.spp_end, W.k_per_wave, W.npix);
    k_raygen<false><<<Lc.grid_raygen, Lc.block_stage, 0, st>>>(P, W);
    for (uint32_t d = 0; d < W.max_depth; ++d) {
        mark(ctx, STAGE_EXTEND);
        launch_extend<false>(st, Lc, S, P, W, d);
        mark(ctx, STAGE_SHADE);
        if (W.sort) enqueue_sort(ctx, S, P, Lc, d, W.sort);
        k_shade<false><<<Lc.grid_shade, Lc.block_shade, 0, st>>>(S, P, W, d);
        if (W.ns > 0) {
            mark(ctx, STAGE_SHADOW);
            launch_shadow<false>(st, Lc, S, P, W, d);
        }
    }
    mark(ctx, STAGE_OTHER);
    k_accumulate<<<Lc.grid_acc, Lc.block_stage, 0, st>>>(P, W);
    k_wave_end<<<1, 32, 0, st>>>(P.ctl, W.max_depth);
    mark(ctx, STAGE_END);
}

// One batch wave: the same stages over paths of several jobs; W.max_depth is
// the deepest job's (shallower jobs stop enqueueing their paths earlier).
void enqueue_wave_batch(pyre_ctx* ctx, const DevScene& S, const PathSoA& P, const WaveParams& W, const Launch& Lc) {
    cudaStream_t st = ctx->stream;
    mark(ctx, STAGE_OTHER);
    k_wave_begin_batch<<<1, 32, 0, st>>>(P.ctl, W.waves);
    k_raygen<true><<<Lc.grid_raygen, Lc.block_stage, 0, st>>>(P, W);
    for (uint32_t d = 0; d < W.max_depth; ++d) {
        mark(ctx, STAGE_EXTEND);
        launch_extend<true>(st, Lc, S, P, W, d);
        mark(ctx, STAGE_SHADE);
        if (W.sort) enqueue_sort(ctx, S, P, Lc, d, W.sort);
        k_shade<true><<<Lc.grid_shade, Lc.block_shade, 0, st>>>(S, P, W, d);
        if (W.ns > 0) {
            mark(ctx, STAGE_SHADOW);
            launch_shadow<true>(st, Lc, S, P, W, d);
        }
    }
    mark(ctx, STAGE_OTHER);
    k_accumulate_batch<<<Lc.grid_acc, Lc.block_stage, 0, st>>>(P, W);
    k_wave_end<<<1, 32, 0, st>>>(P.ctl, W.max_depth);
    mark(ctx, STAGE_END);
}

uint32_t kernels_per_wave(const WaveParams& W) {
    return 4 + W.max_depth * ((W.ns > 0 ? 3 : 2) + (W.sort == PYRE_SORT_TILES ? 1 : W.sort ? 3 : 0));
}

// Largest pixel count of one view: path and pixel indices are 32-bit, and a
// wave holds at least one sample of every pixel.
#define PYRE_MAX_PIXELS (1ull << 31)

// The crop of the render parameters (all zero = the whole image) as
// c = {x0, y0, x1, y1} and its pixel count, computed in 64 bits: crops outside
// the image, empty crops and crops above PYRE_MAX_PIXELS are rejected before
// anything divides by the count.
int resolve_crop(pyre_ctx* ctx, const pyre_render_params& rp, const char* who, uint32_t c[4], uint32_t* npix) {
    if (rp.width == 0 || rp.height == 0) return set_error(ctx, PYRE_ERR_INVALID, std::string(who) + ": image size is zero");
    c[0] = rp.crop[0]; c[1] = rp.crop[1]; c[2] = rp.crop[2]; c[3] = rp.crop[3];
    if (c[0] == 0 && c[1] == 0 && c[2] == 0 && c[3] == 0) { c[2] = rp.width; c[3] = rp.height; }
    if (c[2] > rp.width || c[3] > rp.height || c[0] >= c[2] || c[1] >= c[3])
        return set_error(ctx, PYRE_ERR_INVALID, std::string(who) + ": crop outside the image");
    const uint64_t n = (uint64_t)(c[2] - c[0]) * (uint64_t)(c[3] - c[1]);
    if (n == 0 || n > PYRE_MAX_PIXELS)
        return set_error(ctx, PYRE_ERR_INVALID, std::string(who) + ": crop of " + std::to_string(n) +
                                                    " pixels (at most 2^31 per view)");
    *npix = (uint32_t)n;
    return PYRE_OK;
}

}  // namespace
}  // namespace pyre

using namespace pyre;

static int render_impl(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                       const pyre_render_params* params, pyre_film* film, float4* keep, float* prog = nullptr);

extern "C" {

int pyre_render(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                const pyre_render_params* params, pyre_film* film) {
    NvtxRange nvtx("pyre_render");
    return render_impl(ctx, scene, camera, params, film, nullptr);
}

int pyre_render_progressive(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                            const pyre_render_params* params, float* mean_rgb, int mem) {
    NvtxRange nvtx("pyre_render_progressive");
    if (!ctx || !scene || !camera || !params || !mean_rgb)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_render_progressive: NULL argument");
    if (mem != PYRE_MEM_HOST && mem != PYRE_MEM_DEVICE)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_render_progressive: mem must be PYRE_MEM_HOST or PYRE_MEM_DEVICE");
    uint32_t c[4], npix = 0;
    int rc = resolve_crop(ctx, *params, "pyre_render_progressive", c, &npix);
    if (rc) return rc;
    cudaSetDevice(ctx->device);
    pyre_film none;
    std::memset(&none, 0, sizeof none);
    none.mem = PYRE_MEM_DEVICE;
    if (mem == PYRE_MEM_DEVICE) return render_impl(ctx, scene, camera, params, &none, nullptr, mean_rgb);
    const size_t bytes = (size_t)npix * 3 * sizeof(float);
    rc = ensure_workspace(ctx, ctx->prog_ws, bytes);
    if (rc) return rc;
    float* d = (float*)ctx->prog_ws.ptr;
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(d, mean_rgb, bytes, cudaMemcpyHostToDevice, ctx->stream));
    if ((rc = render_impl(ctx, scene, camera, params, &none, nullptr, d))) return rc;
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(mean_rgb, d, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return PYRE_OK;
}

}  // extern "C"

// The render; with `keep` non-null each path's final radiance is also
// written to keep[(s - spp_begin) * npix + pixel] (pyre_forward). With `prog`
// non-null (device, crop npix x 3) the samples are merged into that running
// radiance mean instead of the film's radiance (pyre_render_progressive).
static int render_impl(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                       const pyre_render_params* params, pyre_film* film, float4* keep, float* prog) {
    if (!ctx || !scene || !camera || !params || !film)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_render: NULL argument");
    cudaSetDevice(ctx->device);
    const pyre_render_params& rp = *params;
    uint32_t c[4], npix = 0;
    int rc = resolve_crop(ctx, rp, "pyre_render", c, &npix);
    if (rc) return rc;
    if (rp.spp_end <= rp.spp_begin) return set_error(ctx, PYRE_ERR_INVALID, "empty sample range");
    if (rp.max_depth > PYRE_MAX_DEPTH) return set_error(ctx, PYRE_ERR_INVALID, "max_depth above 64");
    if (camera->kind > PYRE_CAMERA_THIN_LENS) return set_error(ctx, PYRE_ERR_INVALID, "unknown camera kind");
    if (film->mem != PYRE_MEM_HOST && film->mem != PYRE_MEM_DEVICE)
        return set_error(ctx, PYRE_ERR_INVALID, "film.mem must be PYRE_MEM_HOST or PYRE_MEM_DEVICE");

    WaveParams W;
    std::memset(&W, 0, sizeof W);
    W.cam = make_camera(*camera);
    W.width = rp.width; W.height = rp.height;
    W.cx0 = c[0]; W.cy0 = c[1]; W.cw = c[2] - c[0]; W.ch = c[3] - c[1];
    W.npix = npix;
    W.spp_begin = rp.spp_begin; W.spp_end = rp.spp_end;
    W.max_depth = rp.max_depth; W.min_rr = rp.min_rr_depth;
    W.ns = scene->dev.n_lights + (scene->dev.has_env ? 1u : 0u);
    W.env_cdf = rp.env_sampling == PYRE_ENV_CDF ? 1 : 0;
    W.refill = refill_lanes(&rp);
    W.refill_any = refill_lanes(&rp, true);
    W.sort = sort_kind(rp.sort_by_material, PYRE_SORT_OFF);
    if (W.sort < 0) return set_error(ctx, PYRE_ERR_INVALID, "sort_by_material must be 0, 1, 2 or 3");
    W.prog_mean = prog;
    DevScene D;
    rc = select_bvh(ctx, const_cast<pyre_scene*>(scene), rp.bvh_width, &D, &W.bvh_width);
    if (rc) return rc;
    const uint32_t spp = rp.spp_end - rp.spp_begin;
    uint64_t target = rp.wave_paths ? rp.wave_paths : default_wave_paths(ctx, W.ns, false, false);
    uint64_t K = std::max<uint64_t>(1, target / W.npix);
    K = std::min<uint64_t>(K, spp);
    if ((uint64_t)W.npix * K > (uint64_t)1 << 31) K = std::max<uint64_t>(1, ((uint64_t)1 << 31) / W.npix);
    W.k_per_wave = (uint32_t)K;
    const size_t P = (size_t)W.npix * K;
    const uint32_t waves = (uint32_t)((spp + K - 1) / K);

    size_t film_bytes = (size_t)W.npix * 10 * sizeof(float);
    size_t need = carve_paths(nullptr, P, std::max(W.ns, 1u), W.npix, nullptr);
    rc = ensure_workspace(ctx, ctx->render_ws, need);
    if (rc) return rc;
    PathSoA S;
    carve_paths((char*)ctx->render_ws.ptr, P, std::max(W.ns, 1u), W.npix, &S);
    S.keep_L = keep;
    if (film->mem == PYRE_MEM_HOST && (rc = ensure_workspace(ctx, ctx->io_ws, film_bytes))) return rc;

    const Launch Lc = make_launch<false>(ctx, rp.block_size, W.bvh_width);

    cudaStream_t st = ctx->stream;
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.acc_r, 0, (size_t)W.npix * sizeof(float4), st));
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.acc_a, 0, (size_t)W.npix * sizeof(float4), st));
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.acc_n, 0, (size_t)W.npix * sizeof(float4), st));
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.ctl, 0, sizeof(WaveCtl), st));
    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[0], st));

    ctx->stage_used = 0;
    if (rp.use_graph && !ctx->stage_timing && !keep && !prog) {
        // One wave captured once per configuration, replayed `waves` times.
        char key[256];
        std::snprintf(key, sizeof key, "%llu/%p/%u/%u/%u/%u/%u/%u/%u/%u/%d/r%d/s%d/w%d",
                      (unsigned long long)scene->serial, ctx->render_ws.ptr, W.npix, W.k_per_wave, W.max_depth,
                      W.min_rr, W.ns, W.spp_begin, W.spp_end, W.cx0 + W.cy0 * 65536u, W.env_cdf, W.refill, W.sort,
                      W.bvh_width);
        std::string k2 = std::string(key) + "/" + std::to_string(W.width) + "x" + std::to_string(W.height) + "/b" +
                         std::to_string(Lc.block_stage) + "x" + std::to_string(Lc.block_shade) + "x" +
                         std::to_string(Lc.block_trace);
        // camera bytes are part of the key
        k2.append(reinterpret_cast<const char*>(&W.cam), sizeof(W.cam));
        if (!ctx->wave_graph || ctx->wave_graph_key != k2) {
            if (ctx->wave_graph) { cudaGraphExecDestroy(ctx->wave_graph); ctx->wave_graph = nullptr; }
            cudaGraph_t g;
            PYRE_CUDA_TRY(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            enqueue_wave(ctx, D, S, W, Lc);
            PYRE_CUDA_TRY(ctx, cudaStreamEndCapture(st, &g));
            cudaError_t e = cudaGraphInstantiate(&ctx->wave_graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { ctx->wave_graph = nullptr; return cuda_check(ctx, e, "cudaGraphInstantiate"); }
            ctx->wave_graph_key = k2;
        }
        for (uint32_t w = 0; w < waves; ++w) PYRE_CUDA_TRY(ctx, cudaGraphLaunch(ctx->wave_graph, st));
    } else {
        for (uint32_t w = 0; w < waves; ++w) enqueue_wave(ctx, D, S, W, Lc);
    }
    PYRE_CUDA_TRY(ctx, cudaGetLastError());

    const float inv_spp = 1.0f / (float)spp;
    float* out[4] = {prog ? nullptr : film->radiance, film->albedo, film->normal, film->depth};
    float* dst[4];
    float* staging = (float*)ctx->io_ws.ptr;
    size_t offs[4] = {0, (size_t)W.npix * 3, (size_t)W.npix * 6, (size_t)W.npix * 9};
    for (int c = 0; c < 4; ++c) dst[c] = out[c] ? (film->mem == PYRE_MEM_HOST ? staging + offs[c] : out[c]) : nullptr;
    k_finalize<<<Lc.grid_acc, 256, 0, st>>>(S, W.npix, inv_spp, dst[0], dst[1], dst[2], dst[3]);
    PYRE_CUDA_TRY(ctx, cudaGetLastError());
    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[1], st));
    if (film->mem == PYRE_MEM_HOST) {
        for (int c = 0; c < 4; ++c)
            if (out[c])
                PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(out[c], dst[c], (c == 3 ? 1 : 3) * (size_t)W.npix * sizeof(float),
                                                   cudaMemcpyDeviceToHost, st));
    }
    WaveCtl ctl;
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(&ctl, S.ctl, sizeof ctl, cudaMemcpyDeviceToHost, st));
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if ((rc = take_kernel_error(ctx))) return rc;
    pyre_render_stats& s = ctx->stats;
    std::memset(&s, 0, sizeof s);
    s.samples = ctl.samples;
    s.extend_rays = ctl.extend_rays;
    s.shadow_rays = ctl.shadow_rays;
    s.waves = waves;
    s.kernel_launches = waves * kernels_per_wave(W) + 1;
    cudaEventElapsedTime(&s.ms_total, ctx->ev[0], ctx->ev[1]);
    if (ctx->stage_timing) {
        float acc[4] = {0, 0, 0, 0};
        for (size_t k = 0; k + 1 < ctx->stage_used; ++k) {
            int tag = ctx->stage_tag[k];
            if (tag > STAGE_OTHER) continue;
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ctx->stage_ev[k], ctx->stage_ev[k + 1]);
            acc[tag] += ms;
        }
        s.ms_extend = acc[STAGE_EXTEND];
        s.ms_shade = acc[STAGE_SHADE];
        s.ms_shadow = acc[STAGE_SHADOW];
        s.ms_other = acc[STAGE_OTHER];
    }
    return PYRE_OK;
}

// ----------------------------------------------------------- batch render --
extern "C" int pyre_render_batch(pyre_ctx* ctx, const pyre_scene* scene, const pyre_batch_job* jobs,
                                 uint32_t n_jobs, const pyre_render_params* params) {
    NvtxRange nvtx("pyre_render_batch");
    if (!ctx || !scene || !jobs || n_jobs == 0)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_render_batch: NULL argument or no jobs");
    PYRE_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    if (scene->dev.has_env)
        return set_error(ctx, PYRE_ERR_UNSUPPORTED, "pyre_render_batch: environment maps are not batched");
    const uint32_t wave_paths = params ? params->wave_paths : 0u;
    const bool use_graph = params && params->use_graph && !ctx->stage_timing;

    // ---- job table
    std::vector<DevJob> dj(n_jobs);
    uint64_t total_pix = 0, total_samples = 0, max_npix = 0;
    uint32_t max_depth = 0;
    for (uint32_t j = 0; j < n_jobs; ++j) {
        const pyre_batch_job& jb = jobs[j];
        const std::string tag = "batch job " + std::to_string(j) + ": ";
        if (jb.part >= scene->n_parts) return set_error(ctx, PYRE_ERR_INVALID, tag + "scene part out of range");
        if (jb.width == 0 || jb.height == 0) return set_error(ctx, PYRE_ERR_INVALID, tag + "image size is zero");
        if (jb.spp_end <= jb.spp_begin) return set_error(ctx, PYRE_ERR_INVALID, tag + "empty sample range");
        if (jb.max_depth > PYRE_MAX_DEPTH) return set_error(ctx, PYRE_ERR_INVALID, tag + "max_depth above 64");
        if (jb.camera.kind > PYRE_CAMERA_THIN_LENS) return set_error(ctx, PYRE_ERR_INVALID, tag + "bad camera");
        if (jb.film.mem != PYRE_MEM_HOST && jb.film.mem != PYRE_MEM_DEVICE)
            return set_error(ctx, PYRE_ERR_INVALID, tag + "bad film.mem");
        DevJob& d = dj[j];
        std::memset(&d, 0, sizeof d);
        d.cam = make_camera(jb.camera);
        if ((uint64_t)jb.width * jb.height > PYRE_MAX_PIXELS)
            return set_error(ctx, PYRE_ERR_INVALID, tag + "more than 2^31 pixels");
        d.width = jb.width; d.height = jb.height;
        d.npix = (uint32_t)((uint64_t)jb.width * jb.height);
        d.spp_begin = jb.spp_begin; d.spp_end = jb.spp_end;
        d.max_depth = jb.max_depth; d.min_rr = jb.min_rr_depth;
        d.tlas_root = scene->part_tlas[jb.part];
        d.light_first = scene->part_light[2 * jb.part];
        d.light_count = scene->part_light[2 * jb.part + 1];
        d.acc_base = (uint32_t)total_pix;
        d.inv_spp = 1.0f / (float)(jb.spp_end - jb.spp_begin);
        total_pix += d.npix;
        total_samples += (uint64_t)d.npix * (jb.spp_end - jb.spp_begin);
        max_npix = std::max<uint64_t>(max_npix, d.npix);
        max_depth = std::max(max_depth, jb.max_depth);
    }
    if (total_pix > 0x7fffffffull) return set_error(ctx, PYRE_ERR_INVALID, "pyre_render_batch: too many pixels");

    // ---- wave plan: jobs packed in order, each job's samples in order
    uint64_t cap = wave_paths ? wave_paths : default_wave_paths(ctx, scene->part_light_max, true, false);
    cap = std::min<uint64_t>(std::max<uint64_t>(cap, max_npix), (uint64_t)1 << 31);
    std::vector<DevSeg> segs;
    std::vector<DevWave> waves;
    std::vector<uint32_t> last_wave(n_jobs, 0);  // the wave that completes each job
    DevWave cur{0, 0, 0, 0};
    for (uint32_t j = 0; j < n_jobs; ++j) {
        uint32_t s = jobs[j].spp_begin, remaining = jobs[j].spp_end - jobs[j].spp_begin;
        while (remaining > 0) {
            uint64_t k = std::min<uint64_t>(remaining, (cap - cur.n_paths) / dj[j].npix);
            if (k == 0) {
                waves.push_back(cur);
                cur = DevWave{(uint32_t)segs.size(), 0, 0, 0};
                continue;
            }
            last_wave[j] = (uint32_t)waves.size();
            segs.push_back(DevSeg{j, s, (uint32_t)k, cur.n_paths, cur.n_slots});
            cur.seg_count += 1;
            cur.n_paths += (uint32_t)(k * dj[j].npix);
            cur.n_slots += dj[j].npix;
            s += (uint32_t)k;
            remaining -= (uint32_t)k;
        }
    }
    if (cur.seg_count) waves.push_back(cur);
    uint64_t max_paths = 0;
    for (const DevWave& w : waves) max_paths = std::max<uint64_t>(max_paths, w.n_paths);

    WaveParams W;
    std::memset(&W, 0, sizeof W);
    W.max_depth = max_depth;
    W.ns = scene->part_light_max;
    W.refill = refill_lanes(params);
    W.refill_any = refill_lanes(params, true);
    W.sort = sort_kind(params ? params->sort_by_material : 0u, PYRE_SORT_OFF);
    if (W.sort < 0) return set_error(ctx, PYRE_ERR_INVALID, "sort_by_material must be 0, 1, 2 or 3");
    DevScene D;
    int rc = select_bvh(ctx, const_cast<pyre_scene*>(scene), params ? params->bvh_width : 0u, &D, &W.bvh_width);
    if (rc) return rc;
    const uint32_t ns = std::max(W.ns, 1u);

    // ---- workspace: path state, accumulators, tables, staging film
    const size_t path_bytes = carve_paths(nullptr, max_paths, ns, (uint32_t)total_pix, nullptr, true);
    const size_t job_bytes = dj.size() * sizeof(DevJob), seg_bytes = segs.size() * sizeof(DevSeg),
                 wave_bytes = waves.size() * sizeof(DevWave);
    const size_t stage_bytes = total_pix * 10 * sizeof(float);
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t need = al(path_bytes) + al(job_bytes) + al(seg_bytes) + al(wave_bytes) + al(stage_bytes);
    rc = ensure_workspace(ctx, ctx->render_ws, need);
    if (rc) return rc;
    char* base = (char*)ctx->render_ws.ptr;
    PathSoA S;
    carve_paths(base, max_paths, ns, (uint32_t)total_pix, &S, true);
    DevJob* d_jobs = (DevJob*)(base + al(path_bytes));
    DevSeg* d_segs = (DevSeg*)((char*)d_jobs + al(job_bytes));
    DevWave* d_waves = (DevWave*)((char*)d_segs + al(seg_bytes));
    float* d_stage = (float*)((char*)d_waves + al(wave_bytes));
    W.jobs = d_jobs; W.segs = d_segs; W.waves = d_waves;

    cudaStream_t st = ctx->stream;
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(d_jobs, dj.data(), job_bytes, cudaMemcpyHostToDevice, st));
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(d_segs, segs.data(), seg_bytes, cudaMemcpyHostToDevice, st));
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(d_waves, waves.data(), wave_bytes, cudaMemcpyHostToDevice, st));
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.acc_r, 0, total_pix * sizeof(float4), st));
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.acc_a, 0, total_pix * sizeof(float4), st));
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.acc_n, 0, total_pix * sizeof(float4), st));
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.ctl, 0, sizeof(WaveCtl), st));

    const Launch Lc = make_launch<true>(ctx, params ? params->block_size : 0u, W.bvh_width);

    const uint32_t n_waves = (uint32_t)waves.size();
    // Jobs completed by each wave: [done_lo[w], done_lo[w + 1]) (jobs are packed in order, so their last
    // waves do not decrease).
    std::vector<uint32_t> done_lo(n_waves + 1, n_jobs);
    for (uint32_t j = n_jobs; j-- > 0;) done_lo[last_wave[j]] = j;
    for (uint32_t w = n_waves; w-- > 0;) done_lo[w] = std::min(done_lo[w], done_lo[w + 1]);
    if (!ctx->copy_stream)
        PYRE_CUDA_TRY(ctx, cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
    while (ctx->wave_ev.size() < n_waves) {
        cudaEvent_t e;
        PYRE_CUDA_TRY(ctx, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->wave_ev.push_back(e);
    }

    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[0], st));
    ctx->stage_used = 0;
    if (use_graph) {
        // One wave (its bounce loop) as a graph: every wave runs the same kernels, and the kernels read which
        // segments the current wave holds from the device tables (WaveCtl::wave), so the graph is replayed
        // once per wave.
        std::string key = "batchwave/" + std::to_string(scene->serial) + "/" +
                          std::to_string((uintptr_t)ctx->render_ws.ptr) + "/" + std::to_string(max_depth) + "/" +
                          std::to_string(max_paths) + "/" + std::to_string(total_pix) + "/" +
                          std::to_string(dj.size()) + "/" + std::to_string(segs.size()) + "/b" +
                          std::to_string(Lc.block_stage) + "x" + std::to_string(Lc.block_shade) + "x" +
                          std::to_string(Lc.block_trace) + "/r" + std::to_string(W.refill) + "/s" +
                          std::to_string(W.sort) + "/w" + std::to_string(W.bvh_width);
        if (!ctx->wave_graph || ctx->wave_graph_key != key) {
            if (ctx->wave_graph) { cudaGraphExecDestroy(ctx->wave_graph); ctx->wave_graph = nullptr; }
            cudaGraph_t g;
            PYRE_CUDA_TRY(ctx, cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            enqueue_wave_batch(ctx, D, S, W, Lc);
            PYRE_CUDA_TRY(ctx, cudaStreamEndCapture(st, &g));
            cudaError_t e = cudaGraphInstantiate(&ctx->wave_graph, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { ctx->wave_graph = nullptr; return cuda_check(ctx, e, "cudaGraphInstantiate"); }
            ctx->wave_graph_key = key;
        }
    }
    // Every wave is enqueued first; after the wave that completes some jobs, their films are finalized and
    // an event marks them done. The copies to the callers' films then run on a second stream while the GPU
    // renders the waves that follow, which per-view calls (one synchronous render each) cannot overlap.
    uint32_t finalizes = 0;
    for (uint32_t w = 0; w < n_waves; ++w) {
        if (use_graph) PYRE_CUDA_TRY(ctx, cudaGraphLaunch(ctx->wave_graph, st));
        else enqueue_wave_batch(ctx, D, S, W, Lc);
        const uint32_t j0 = done_lo[w], j1 = done_lo[w + 1];
        if (j0 < j1) {
            const uint32_t a0 = dj[j0].acc_base, a1 = dj[j1 - 1].acc_base + dj[j1 - 1].npix;
            k_finalize_batch<<<Lc.grid_acc, 256, 0, st>>>(S, d_jobs, n_jobs, (uint32_t)total_pix, a0, a1, d_stage);
            ++finalizes;
            PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->wave_ev[w], st));
        }
    }
    PYRE_CUDA_TRY(ctx, cudaGetLastError());
    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[1], st));
    cudaStream_t cst = ctx->copy_stream;
    for (uint32_t w = 0; w < n_waves; ++w) {
        if (done_lo[w] == done_lo[w + 1]) continue;
        PYRE_CUDA_TRY(ctx, cudaStreamWaitEvent(cst, ctx->wave_ev[w], 0));
        for (uint32_t j = done_lo[w]; j < done_lo[w + 1]; ++j) {
            const pyre_film& f = jobs[j].film;
            const cudaMemcpyKind kind = f.mem == PYRE_MEM_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
            const size_t a = dj[j].acc_base, n = dj[j].npix;
            float* outs[4] = {f.radiance, f.albedo, f.normal, f.depth};
            for (int c = 0; c < 4; ++c) {
                if (!outs[c]) continue;
                const size_t comps = c == 3 ? 1 : 3;
                const float* src = d_stage + (size_t)c * 3 * total_pix + comps * a;
                PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(outs[c], src, comps * n * sizeof(float), kind, cst));
            }
        }
    }
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(cst));
    WaveCtl ctl;
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(&ctl, S.ctl, sizeof ctl, cudaMemcpyDeviceToHost, st));
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if ((rc = take_kernel_error(ctx))) return rc;
    pyre_render_stats& s = ctx->stats;
    std::memset(&s, 0, sizeof s);
    s.samples = ctl.samples;
    s.extend_rays = ctl.extend_rays;
    s.shadow_rays = ctl.shadow_rays;
    s.waves = n_waves;
    s.kernel_launches = n_waves * kernels_per_wave(W) + finalizes;
    cudaEventElapsedTime(&s.ms_total, ctx->ev[0], ctx->ev[1]);
    return PYRE_OK;
}

// --------------------------------------------------- render without malloc --
// Path state for pyre_render_noalloc: one static array per device that loads
// the library, used in place of the context's cudaMalloc'd workspace.
namespace pyre {
static __device__ __align__(256) unsigned char g_noalloc_scratch[PYRE_NOALLOC_SCRATCH_BYTES];

namespace {
std::mutex g_noalloc_mu;
void* g_noalloc_addr[256] = {};

// Device address of the static array on ctx->device (looked up once per
// device, with that device current).
int noalloc_scratch(pyre_ctx* ctx, void** out) {
    if (ctx->device < 0 || ctx->device >= 256) return set_error(ctx, PYRE_ERR_INVALID, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    if (!g_noalloc_addr[ctx->device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_check(ctx, e, "cudaGetSymbolAddress(noalloc scratch)");
        g_noalloc_addr[ctx->device] = p;
    }
    *out = g_noalloc_addr[ctx->device];
    return PYRE_OK;
}
}  // namespace
}  // namespace pyre

extern "C" int pyre_render_noalloc(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                                   const pyre_render_params* params, pyre_film* film) {
    NvtxRange nvtx("pyre_render_noalloc");
    if (!ctx || !scene || !camera || !params || !film)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_render_noalloc: NULL argument");
    PYRE_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const pyre_render_params& rp = *params;
    if (film->mem != PYRE_MEM_DEVICE)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_render_noalloc: the film must be device memory");
    uint32_t c[4], npix = 0;
    int rc = resolve_crop(ctx, rp, "pyre_render_noalloc", c, &npix);
    if (rc) return rc;
    if (rp.spp_end <= rp.spp_begin) return set_error(ctx, PYRE_ERR_INVALID, "empty sample range");
    if (rp.max_depth > PYRE_MAX_DEPTH) return set_error(ctx, PYRE_ERR_INVALID, "max_depth above 64");
    if (camera->kind > PYRE_CAMERA_THIN_LENS) return set_error(ctx, PYRE_ERR_INVALID, "unknown camera kind");

    WaveParams W;
    std::memset(&W, 0, sizeof W);
    W.cam = make_camera(*camera);
    W.width = rp.width; W.height = rp.height;
    W.cx0 = c[0]; W.cy0 = c[1]; W.cw = c[2] - c[0]; W.ch = c[3] - c[1];
    W.npix = npix;
    W.spp_begin = rp.spp_begin; W.spp_end = rp.spp_end;
    W.max_depth = rp.max_depth; W.min_rr = rp.min_rr_depth;
    W.ns = scene->dev.n_lights + (scene->dev.has_env ? 1u : 0u);
    W.env_cdf = rp.env_sampling == PYRE_ENV_CDF ? 1 : 0;
    W.refill = refill_lanes(&rp);
    W.refill_any = refill_lanes(&rp, true);
    W.sort = sort_kind(rp.sort_by_material, PYRE_SORT_OFF);
    if (W.sort < 0) return set_error(ctx, PYRE_ERR_INVALID, "sort_by_material must be 0, 1, 2 or 3");
    DevScene D;
    rc = select_bvh(ctx, const_cast<pyre_scene*>(scene), rp.bvh_width, &D, &W.bvh_width, false);
    if (rc) return rc;
    const uint32_t ns = std::max(W.ns, 1u);
    const size_t cap = PYRE_NOALLOC_SCRATCH_BYTES;
    if (carve_paths(nullptr, W.npix, ns, W.npix, nullptr) > cap) {
        uint64_t lo = 1, hi = W.npix;  // largest pixel count that fits one sample per pixel
        while (lo < hi) {
            uint64_t mid = (lo + hi + 1) / 2;
            if (carve_paths(nullptr, mid, ns, (uint32_t)mid, nullptr) <= cap) lo = mid; else hi = mid - 1;
        }
        return set_error(ctx, PYRE_ERR_INVALID,
                         "pyre_render_noalloc: crop of " + std::to_string(W.npix) + " pixels exceeds the " +
                             std::to_string(cap >> 20) + " MiB static path-state array (at most " +
                             std::to_string(lo) + " pixels with " + std::to_string(W.ns) +
                             " NEE slots per path); render the image as smaller crop tiles");
    }
    const uint32_t spp = rp.spp_end - rp.spp_begin;
    uint64_t target = rp.wave_paths ? rp.wave_paths : (uint64_t)8 << 20;
    uint64_t K = std::min<uint64_t>(std::max<uint64_t>(1, target / W.npix), spp);
    if (carve_paths(nullptr, (size_t)W.npix * K, ns, W.npix, nullptr) > cap) {
        uint64_t lo = 1, hi = K - 1;  // largest K whose wave fits (K = 1 fits, checked above)
        while (lo < hi) {
            const uint64_t mid = (lo + hi + 1) / 2;
            if (carve_paths(nullptr, (size_t)W.npix * mid, ns, W.npix, nullptr) <= cap) lo = mid; else hi = mid - 1;
        }
        K = lo;
    }
    W.k_per_wave = (uint32_t)K;
    const uint32_t waves = (uint32_t)((spp + K - 1) / K);

    void* scratch = nullptr;
    rc = noalloc_scratch(ctx, &scratch);
    if (rc) return rc;
    PathSoA S;
    carve_paths((char*)scratch, (size_t)W.npix * K, ns, W.npix, &S);

    const Launch Lc = make_launch<false>(ctx, rp.block_size, W.bvh_width);

    cudaStream_t st = ctx->stream;
    // The array keeps the previous call's contents: clear the sums and counters.
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.acc_r, 0, (size_t)W.npix * sizeof(float4), st));
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.acc_a, 0, (size_t)W.npix * sizeof(float4), st));
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.acc_n, 0, (size_t)W.npix * sizeof(float4), st));
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.ctl, 0, sizeof(WaveCtl), st));
    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[0], st));
    const int timing = ctx->stage_timing;
    ctx->stage_timing = 0;  // stage timing would create events
    for (uint32_t w = 0; w < waves; ++w) enqueue_wave(ctx, D, S, W, Lc);
    ctx->stage_timing = timing;
    PYRE_CUDA_TRY(ctx, cudaGetLastError());
    k_finalize<<<Lc.grid_acc, 256, 0, st>>>(S, W.npix, 1.0f / (float)spp, film->radiance, film->albedo, film->normal,
                                              film->depth);
    PYRE_CUDA_TRY(ctx, cudaGetLastError());
    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[1], st));
    WaveCtl ctl;
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(&ctl, S.ctl, sizeof ctl, cudaMemcpyDeviceToHost, st));
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if ((rc = take_kernel_error(ctx))) return rc;
    pyre_render_stats& s = ctx->stats;
    std::memset(&s, 0, sizeof s);
    s.samples = ctl.samples;
    s.extend_rays = ctl.extend_rays;
    s.shadow_rays = ctl.shadow_rays;
    s.waves = waves;
    s.kernel_launches = waves * kernels_per_wave(W) + 1;
    cudaEventElapsedTime(&s.ms_total, ctx->ev[0], ctx->ev[1]);
    return PYRE_OK;
}

template <bool ANY>
static void launch_intersect(pyre_ctx* ctx, const DevScene& D, const QueryRays& q, uint32_t n, int width) {
    cudaStream_t st = ctx->stream;
    const int refill = ANY ? PYRE_DEFAULT_REFILL_ANY : PYRE_DEFAULT_REFILL;
    if (width == 8) {
        k_intersect<ANY, 8><<<grid_for(ctx, k_intersect<ANY, 8>, 128), 128, 0, st>>>(D, q, n, ctx->d_counter, refill);
    } else if (width == 4) {
        k_intersect<ANY, 4><<<grid_for(ctx, k_intersect<ANY, 4>, 128), 128, 0, st>>>(D, q, n, ctx->d_counter, refill);
    } else {
        k_intersect<ANY, 2><<<grid_for(ctx, k_intersect<ANY, 2>, 128), 128, 0, st>>>(D, q, n, ctx->d_counter, refill);
    }
}

extern "C" {

static int intersect_impl(pyre_ctx* ctx, const pyre_scene* scene, const pyre_rays* rays, uint64_t n, pyre_hits* hits,
                          uint8_t* occluded, int mem, bool any) {
    NvtxRange nvtx(any ? "pyre_intersect_any" : "pyre_intersect_closest");
    if (!ctx || !scene || !rays) return set_error(ctx, PYRE_ERR_INVALID, "intersect: NULL argument");
    if (!rays->origin || !rays->direction || !rays->t_min || !rays->t_max)
        return set_error(ctx, PYRE_ERR_INVALID, "intersect: ray arrays missing");
    if (any ? !occluded : (!hits || !hits->kind || !hits->instance || !hits->triangle || !hits->t || !hits->u || !hits->v))
        return set_error(ctx, PYRE_ERR_INVALID, "intersect: output arrays missing");
    if (mem != PYRE_MEM_HOST && mem != PYRE_MEM_DEVICE) return set_error(ctx, PYRE_ERR_INVALID, "intersect: bad mem");
    if (n == 0) return PYRE_OK;
    if (n > 0x7fffffffull) return set_error(ctx, PYRE_ERR_INVALID, "intersect: more than 2^31-1 rays");
    cudaSetDevice(ctx->device);
    DevScene D;
    int width = 2;
    if (int rc0 = select_bvh(ctx, const_cast<pyre_scene*>(scene), 0u, &D, &width)) return rc0;
    cudaStream_t st = ctx->stream;
    const float *org = rays->origin, *dir = rays->direction, *tmin = rays->t_min, *tmax = rays->t_max,
                *time = rays->time;
    int32_t *kind = nullptr, *inst = nullptr, *tri = nullptr;
    float *tt = nullptr, *uu = nullptr, *vv = nullptr;
    uint8_t* occ = occluded;
    if (!any) { kind = hits->kind; inst = hits->instance; tri = hits->triangle; tt = hits->t; uu = hits->u; vv = hits->v; }
    if (mem == PYRE_MEM_HOST) {
        size_t in_bytes = n * (time ? 9 : 8) * sizeof(float);
        size_t out_bytes = any ? n : n * 6 * sizeof(float);
        int rc = ensure_workspace(ctx, ctx->io_ws, in_bytes + out_bytes + 1024);
        if (rc) return rc;
        char* b = (char*)ctx->io_ws.ptr;
        float* d_org = (float*)b;
        float* d_dir = d_org + 3 * n;
        float* d_tmin = d_dir + 3 * n;
        float* d_tmax = d_tmin + n;
        float* d_time = time ? d_tmax + n : nullptr;
        char* ob = (char*)(d_tmax + n + (time ? n : 0));
        PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(d_org, org, 3 * n * sizeof(float), cudaMemcpyHostToDevice, st));
        PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(d_dir, dir, 3 * n * sizeof(float), cudaMemcpyHostToDevice, st));
        PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(d_tmin, tmin, n * sizeof(float), cudaMemcpyHostToDevice, st));
        PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(d_tmax, tmax, n * sizeof(float), cudaMemcpyHostToDevice, st));
        if (time) PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(d_time, time, n * sizeof(float), cudaMemcpyHostToDevice, st));
        org = d_org; dir = d_dir; tmin = d_tmin; tmax = d_tmax; time = d_time;
        if (any) occ = (uint8_t*)ob;
        else {
            kind = (int32_t*)ob; inst = kind + n; tri = inst + n;
            tt = (float*)(tri + n); uu = tt + n; vv = uu + n;
        }
    }
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(ctx->d_counter, 0, sizeof(unsigned int), st));
    QueryRays q{};
    q.org = org; q.dir = dir; q.tmin = tmin; q.tmax = tmax; q.time = time;
    if (any) q.occluded = occ;
    else { q.kind = kind; q.inst = inst; q.tri = tri; q.tt = tt; q.uu = uu; q.vv = vv; }
    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[0], st));
    if (any) launch_intersect<true>(ctx, D, q, (uint32_t)n, width);
    else launch_intersect<false>(ctx, D, q, (uint32_t)n, width);
    PYRE_CUDA_TRY(ctx, cudaGetLastError());
    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[1], st));
    if (mem == PYRE_MEM_HOST) {
        if (any) PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(occluded, occ, n, cudaMemcpyDeviceToHost, st));
        else {
            PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(hits->kind, kind, n * 4, cudaMemcpyDeviceToHost, st));
            PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(hits->instance, inst, n * 4, cudaMemcpyDeviceToHost, st));
            PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(hits->triangle, tri, n * 4, cudaMemcpyDeviceToHost, st));
            PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(hits->t, tt, n * 4, cudaMemcpyDeviceToHost, st));
            PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(hits->u, uu, n * 4, cudaMemcpyDeviceToHost, st));
            PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(hits->v, vv, n * 4, cudaMemcpyDeviceToHost, st));
        }
    }
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if (int rc = take_kernel_error(ctx)) return rc;
    // statistics: the query kernel's device time and its ray count
    pyre_render_stats& s = ctx->stats;
    std::memset(&s, 0, sizeof s);
    (any ? s.shadow_rays : s.extend_rays) = n;
    s.kernel_launches = 1;
    cudaEventElapsedTime(&s.ms_total, ctx->ev[0], ctx->ev[1]);
    return PYRE_OK;
}

int pyre_intersect_closest(pyre_ctx* ctx, const pyre_scene* scene, const pyre_rays* rays, uint64_t n, pyre_hits* hits,
                           int mem) {
    return intersect_impl(ctx, scene, rays, n, hits, nullptr, mem, false);
}

int pyre_intersect_any(pyre_ctx* ctx, const pyre_scene* scene, const pyre_rays* rays, uint64_t n, uint8_t* occluded,
                       int mem) {
    return intersect_impl(ctx, scene, rays, n, nullptr, occluded, mem, true);
}

}  // extern "C"

// ---------------------------------------------------- forward / backward --
// Path-replay adjoint (no reference counterpart: the reference has no
// differentiation). pyre_forward renders like pyre_render and keeps every
// path's final radiance L_total in the context. pyre_backward replays the
// same waves (same kernels, seeds, draws and decisions; k_shade<false, true>
// adds the derivatives) under the detached-sampling convention: only BSDF
// values and emitted radiance carry derivatives. NEE and emission terms are
// differentiated where they arise (NEE ones parked with the radiance and
// dropped by the shadow stage when occluded); the BSDF-sample term of vertex
// d uses beta_{d+1} * R_{d+1} = L_total - L_so_far, exact because the replay
// sums contributions in the forward's order.
namespace {
std::string tape_key(const pyre_scene* scene, const pyre_camera_desc* camera, const pyre_render_params& rp) {
    std::string k = std::to_string(scene->serial) + "/";
    k.append(reinterpret_cast<const char*>(camera), sizeof *camera);
    const uint32_t f[] = {rp.width, rp.height, rp.spp_begin, rp.spp_end, rp.max_depth, rp.min_rr_depth,
                          rp.crop[0], rp.crop[1], rp.crop[2], rp.crop[3], rp.env_sampling};
    k.append(reinterpret_cast<const char*>(f), sizeof f);
    return k;
}
int forward_impl(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                 const pyre_render_params* params, pyre_film* film) {
    const pyre_render_params& rp = *params;
    uint32_t c[4], npix = 0;
    int rc = resolve_crop(ctx, rp, "pyre_forward", c, &npix);
    if (rc) return rc;
    if (rp.spp_end <= rp.spp_begin) return set_error(ctx, PYRE_ERR_INVALID, "empty sample range");
    const uint64_t paths = (uint64_t)npix * (rp.spp_end - rp.spp_begin);
    if (paths > ((uint64_t)1 << 40))
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_forward: more than 2^40 paths to keep for the adjoint");
    rc = ensure_workspace(ctx, ctx->tape_ws, std::max<uint64_t>(paths, 1) * sizeof(float4));
    if (rc) return rc;
    ctx->tape_key.clear();
    rc = render_impl(ctx, scene, camera, params, film, (float4*)ctx->tape_ws.ptr);
    if (rc == PYRE_OK) ctx->tape_key = tape_key(scene, camera, rp);
    return rc;
}
}  // namespace

extern "C" int pyre_forward(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                            const pyre_render_params* params, pyre_film* film) {
    NvtxRange nvtx("pyre_forward");
    if (!ctx || !scene || !camera || !params || !film)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_forward: NULL argument");
    return forward_impl(ctx, scene, camera, params, film);
}

extern "C" int pyre_backward(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                             const pyre_render_params* params, const float* d_loss_d_image, int image_mem,
                             pyre_gradients* grads) {
    NvtxRange nvtx("pyre_backward");
    if (!ctx || !scene || !camera || !params || !d_loss_d_image || !grads)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_backward: NULL argument");
    PYRE_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const pyre_render_params& rp = *params;
    uint32_t c[4], npix = 0;
    int rc = resolve_crop(ctx, rp, "pyre_backward", c, &npix);
    if (rc) return rc;
    if (rp.spp_end <= rp.spp_begin) return set_error(ctx, PYRE_ERR_INVALID, "empty sample range");
    if (rp.max_depth > PYRE_MAX_DEPTH) return set_error(ctx, PYRE_ERR_INVALID, "max_depth above 64");
    if (scene->n_parts != 1) return set_error(ctx, PYRE_ERR_UNSUPPORTED, "pyre_backward: batched scenes");
    if (camera->kind > PYRE_CAMERA_THIN_LENS) return set_error(ctx, PYRE_ERR_INVALID, "unknown camera kind");
    if (image_mem != PYRE_MEM_HOST && image_mem != PYRE_MEM_DEVICE)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_backward: bad image_mem");
    if (grads->mem != PYRE_MEM_HOST && grads->mem != PYRE_MEM_DEVICE)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_backward: bad grads.mem");
    // L_total of every path: kept by pyre_forward with the same arguments, or recomputed now
    if (ctx->tape_key != tape_key(scene, camera, rp)) {
        pyre_film none;
        std::memset(&none, 0, sizeof none);
        none.mem = PYRE_MEM_DEVICE;
        if ((rc = forward_impl(ctx, scene, camera, params, &none))) return rc;
    }

    WaveParams W;
    std::memset(&W, 0, sizeof W);
    W.cam = make_camera(*camera);
    W.width = rp.width; W.height = rp.height;
    W.cx0 = c[0]; W.cy0 = c[1]; W.cw = c[2] - c[0]; W.ch = c[3] - c[1];
    W.npix = npix;
    W.spp_begin = rp.spp_begin; W.spp_end = rp.spp_end;
    W.max_depth = rp.max_depth; W.min_rr = rp.min_rr_depth;
    W.ns = scene->dev.n_lights + (scene->dev.has_env ? 1u : 0u);
    W.env_cdf = rp.env_sampling == PYRE_ENV_CDF ? 1 : 0;
    W.refill = refill_lanes(&rp);
    W.refill_any = refill_lanes(&rp, true);
    // The adjoint shade is bound by instruction fetches: warps of one
    // material run one branch of the BSDF and gradient code. Sorting the
    // whole live-path queue by material is the backward's default: backward
    // 20.0 against 22.2 ms on the 512x512 differentiable-render problem, the
    // same gradients; sorting within tiles (the render default) gave 20.5.
    W.sort = sort_kind(rp.sort_by_material, PYRE_SORT_QUEUE);
    if (W.sort < 0) return set_error(ctx, PYRE_ERR_INVALID, "sort_by_material must be 0, 1, 2 or 3");
    DevScene D;
    if ((rc = select_bvh(ctx, const_cast<pyre_scene*>(scene), rp.bvh_width, &D, &W.bvh_width))) return rc;
    const uint32_t spp = rp.spp_end - rp.spp_begin;
    uint64_t K = std::max<uint64_t>(
        1, (rp.wave_paths ? rp.wave_paths : default_wave_paths(ctx, W.ns, false, true)) / W.npix);
    K = std::min<uint64_t>(K, spp);
    if ((uint64_t)W.npix * K > (uint64_t)1 << 31) K = std::max<uint64_t>(1, ((uint64_t)1 << 31) / W.npix);
    W.k_per_wave = (uint32_t)K;
    const size_t P = (size_t)W.npix * K;
    const uint32_t waves = (uint32_t)((spp + K - 1) / K);

    const uint32_t n_mat = scene->dev.n_materials;
    const size_t mat_bytes = (size_t)n_mat * PYRE_NPARAM * sizeof(double);
    const size_t env_elems = scene->dev.has_env ? (size_t)scene->dev.env.width * scene->dev.env.height * 3 : 0;
    const size_t img_bytes = (size_t)W.npix * 3 * sizeof(float);
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t path_bytes = carve_paths(nullptr, P, std::max(W.ns, 1u), W.npix, nullptr, false, true);
    if ((rc = ensure_workspace(ctx, ctx->render_ws, path_bytes))) return rc;
    if ((rc = ensure_workspace(ctx, ctx->io_ws, al(mat_bytes) + al(env_elems * 4) + al(img_bytes) + 256))) return rc;
    PathSoA S;
    carve_paths((char*)ctx->render_ws.ptr, P, std::max(W.ns, 1u), W.npix, &S, false, true);
    S.keep_L = (float4*)ctx->tape_ws.ptr;
    char* b = (char*)ctx->io_ws.ptr;
    double* d_mat = grads->mem == PYRE_MEM_DEVICE && grads->materials ? grads->materials : (double*)b;
    float* d_env = grads->mem == PYRE_MEM_DEVICE && grads->env ? grads->env : (float*)(b + al(mat_bytes));
    const float* d_img = d_loss_d_image;
    cudaStream_t st = ctx->stream;
    if (image_mem == PYRE_MEM_HOST) {
        float* tmp = (float*)(b + al(mat_bytes) + al(env_elems * 4));
        PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(tmp, d_loss_d_image, img_bytes, cudaMemcpyHostToDevice, st));
        d_img = tmp;
    }
    if (mat_bytes) PYRE_CUDA_TRY(ctx, cudaMemsetAsync(d_mat, 0, mat_bytes, st));
    if (env_elems && grads->env) PYRE_CUDA_TRY(ctx, cudaMemsetAsync(d_env, 0, env_elems * 4, st));
    W.dl_di = d_img;
    W.inv_spp = 1.0f / (float)spp;
    W.mat_grad = d_mat;
    W.env_grad = (env_elems && grads->env) ? d_env : nullptr;
    W.n_mat = n_mat;
    W.env_cache = W.env_grad ? 1 : 0;
    const size_t mat_smem = grad_smem_bytes(W.env_cache, mat_bytes) <= 48 * 1024 ? mat_bytes : 0;
    W.smem_grad = mat_smem ? 1 : 0;
    const size_t smem = grad_smem_bytes(W.env_cache, mat_smem);

    const Launch Lc = make_launch<false>(ctx, rp.block_size, W.bvh_width);
    const int grid_adj = grid_for(ctx, k_shade<false, true>, Lc.block_stage, smem);
    const int grid_acc = grid_for(ctx, k_accumulate_adjoint, Lc.block_stage, smem);
    PYRE_CUDA_TRY(ctx, cudaMemsetAsync(S.ctl, 0, sizeof(WaveCtl), st));
    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[0], st));
    for (uint32_t w = 0; w < waves; ++w) {
        k_wave_begin<<<1, 32, 0, st>>>(S.ctl, W.spp_begin, W.spp_end, W.k_per_wave, W.npix);
        k_raygen<false><<<Lc.grid_raygen, Lc.block_stage, 0, st>>>(S, W);
        for (uint32_t d = 0; d < W.max_depth; ++d) {
            launch_extend<false>(st, Lc, D, S, W, d);
            if (W.sort) enqueue_sort(ctx, D, S, Lc, d, W.sort);
            k_shade<false, true><<<grid_adj, Lc.block_stage, smem, st>>>(D, S, W, d);
            if (W.ns > 0) launch_shadow<false>(st, Lc, D, S, W, d);
        }
        k_accumulate_adjoint<<<grid_acc, Lc.block_stage, smem, st>>>(D, S, W);
        k_wave_end<<<1, 32, 0, st>>>(S.ctl, W.max_depth);
    }
    PYRE_CUDA_TRY(ctx, cudaGetLastError());
    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[1], st));
    if (grads->mem == PYRE_MEM_HOST) {
        if (grads->materials && mat_bytes)
            PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(grads->materials, d_mat, mat_bytes, cudaMemcpyDeviceToHost, st));
        if (grads->env && env_elems)
            PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(grads->env, d_env, env_elems * 4, cudaMemcpyDeviceToHost, st));
    }
    WaveCtl ctl;
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(&ctl, S.ctl, sizeof ctl, cudaMemcpyDeviceToHost, st));
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if ((rc = take_kernel_error(ctx))) return rc;
    pyre_render_stats& s = ctx->stats;
    std::memset(&s, 0, sizeof s);
    s.samples = ctl.samples;
    s.extend_rays = ctl.extend_rays;
    s.shadow_rays = ctl.shadow_rays;
    s.waves = waves;
    s.kernel_launches = waves * kernels_per_wave(W);
    cudaEventElapsedTime(&s.ms_total, ctx->ev[0], ctx->ev[1]);
    return PYRE_OK;
}
