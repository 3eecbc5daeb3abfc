// device_scene.cuh — scene layout in HBM and ray traversal (closest / any hit).
//
// Layout (all arrays device-resident, built once by pyre_scene_upload):
//   nodes  GpuNode[]    64-B binary nodes: every mesh BVH (collapsed from the
//                       reference BVH2), then the top-level BVH over instances
//   tris   float4[3*T]  per triangle slot, in BVH leaf order:
//                       (v0.xyz, original triangle id as bits), (e1.xyz, 0), (e2.xyz, 0)
//                       with e1 = v1 - v0, e2 = v2 - v0 rounded exactly as
//                       moller_trumbore computes them (mesh.rs:153-157)
//   inst   DevInstance[] instances in top-level-leaf order
//   index  uint32[3*T]  mesh index buffers rebased to global vertex ids
//   slot_normals float4[3*T] per triangle slot, its three vertex normals (for shading)
//   normal float[3*V]   vertex normals (meshes without normals use e1 x e2)
#pragma once
#include <cuda_runtime.h>
#include "pyre_math.cuh"

#ifndef PYRE_WIDE_FIELDS
#define PYRE_WIDE_FIELDS 8  // fields of a wide node: 6 box planes, child, count
#endif

namespace pyre {

struct alignas(16) DevInstance {
    float lo[3];  // BLAS root box (the reference tests it first, bvh.rs:103-110)
    int32_t blas_root;  // device node index, -1 for an empty mesh
    float hi[3];
    int32_t has_motion;
    float off0[3];
    int32_t orig_id;    // index in Scene::primitives
    float off1[3];
    int32_t mesh;
    uint32_t material;
    uint32_t index_base;   // first index (3 per triangle) of the mesh in `index`
    int32_t normal_base;   // first vertex of the mesh's normals, -1 if none
    uint32_t tri_count;
};

struct alignas(16) DevMaterial {
    float base[3];
    uint32_t kind;
    float metallic, roughness, specular, pad;
};

struct DevQuadLight {
    f3 p0, edge_u, edge_v, crs, normal, emission;
    float inv_cross_len_sq, area;
};

struct DevEnv {
    uint32_t width, height;
    float intensity;
    const float4* pixels;      // w*h, rgb + pad
    const float* marg_cdf;     // h+1
    const float* cond_cdf;     // h*(w+1)
    const float* marg_pdf;     // h: (cdf[b+1]-cdf[b])*h
    const float* cond_pdf;     // h*w
    const float2* marg_alias;  // h: (prob, alias as bits)
    const float2* cond_alias;  // h*w
};

struct DevScene {
    const float4* nodes;   // GpuNode as 4 float4
    const float4* tris;
    const DevInstance* inst;
    uint32_t n_inst;
    int32_t tlas_root;     // -1: no geometry
    const uint32_t* index;
    const float* normal;
    const float4* slot_normals;  // 3 per triangle slot: its vertex normals (xyz, 0)
    const DevMaterial* materials;
    uint32_t n_materials;
    const DevQuadLight* lights;
    uint32_t n_lights;
    int has_env;
    DevEnv env;
    int* error_flag;       // set to PYRE_ERR_OVERFLOW by a kernel that hit a limit
    // sub-scenes of a batch upload (one part for an ordinary scene)
    const int32_t* part_tlas;    // top-level root per part
    const uint32_t* part_light;  // (first light, light count) per part
    uint32_t n_parts;
    // wide BVH of the instances (traversals with WIDTH 4 or 8; the top level
    // stays binary): wide nodes (8 fields x WIDTH floats each) and the wide
    // root of each instance slot
    const float4* wnodes;
    const int32_t* wroot;
};

struct TraceRay {
    f3 o, d;
    float tmin, tmax, time;
    uint32_t job;  // batched rendering: the ray's job (set and read by the ray source only)
};

struct TraceHit {
    float t, u, v;
    int32_t inst;  // instance slot (device order); -1 = no hit
    int32_t tri;   // triangle slot
    int32_t light; // quad light index when the closest hit is a light, else -1
};

#define PYRE_STACK 64
// lanes of a warp that may still be looking for a leaf when the leaf phase
// starts, for closest-hit and any-hit traversal
// (with two node steps per vote: 12 and 16 against 8 and 12 gave 702.0 and
// 702.7 against 701.0 Msamples/s one at a time; 6 and 8 gave 696.5 and 696.8.
// With instances entered from the top-level step and 9 closest-hit blocks,
// 10 closest-hit lanes measured 748.3 against 746.2 for 12, and 8 748.1.
// Once closest-hit lanes stopped at their first leaf, 16 lanes measured
// 758.8 against 755.6 for 10, 750.7 for 20 and 741.1 for 24)
#ifndef PYRE_LEAF_WAIT_CLOSEST
#define PYRE_LEAF_WAIT_CLOSEST 16
#endif
#ifndef PYRE_LEAF_WAIT_ANY
#define PYRE_LEAF_WAIT_ANY 16
#endif
// Node steps a lane takes between two warp votes of the inner phase. Each
// vote (a ballot, a population count and an any) costs issue slots; taking
// two steps per vote measured 701.8 against 681.0 Msamples/s on the 1080p
// studio frame (extend 104.0 against 109.4 ms), three 700.6. With instances
// entered from the top-level step, three measured 751.3 against 746.4 for
// two (extend 93.9 against 94.9 ms); with 256-bit node loads, four measured
// 768.5 against 763.4 for three. Films are bit-identical for every setting.
#ifndef PYRE_STEPS_PER_VOTE
#define PYRE_STEPS_PER_VOTE 4
#endif

// Binary node fetch: one 64-B node as two 256-bit loads (sm_100+ `ld.v8`;
// nodes are 64-B aligned) instead of four 128-bit ones, so a node step issues
// two load instructions. The traversal is issue-bound: 763.4 against 749.8
// Msamples/s on the 1080p studio frame (extend 92.1 against 94.0 ms, shadow
// 33.2 against 34.5 ms), films bit-identical.
#ifndef PYRE_LD256
#define PYRE_LD256 1
#endif
__device__ __forceinline__ void ldg_256(const float4* p, float4& a, float4& b) {
    asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}

// 32-B path-state records with one streaming (evict-first) 256-bit load or
// store each; p must be 32-B aligned.
__device__ __forceinline__ void ldcs_256(const float4* p, float4& a, float4& b) {
    asm("ld.global.cs.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
        : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
        : "l"(p));
}
__device__ __forceinline__ void stcs_256(float4* p, const float4& a, const float4& b) {
    asm volatile("st.global.cs.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
                 :: "l"(p), "f"(a.x), "f"(a.y), "f"(a.z), "f"(a.w), "f"(b.x), "f"(b.y), "f"(b.z), "f"(b.w)
                 : "memory");
}

// Rust-order slab test (bvh.rs:146-153): t1/t2 per axis, max of mins vs
// t_min, min of maxes vs t_max, hit iff tmin <= tmax. Returns the entry.
__device__ __forceinline__ bool slab(float lox, float hix, float loy, float hiy, float loz, float hiz,
                                     const f3& o, const f3& inv, float tmin_ray, float tmax_cur, float* entry) {
    float t1x = (lox - o.x) * inv.x, t2x = (hix - o.x) * inv.x;
    float t1y = (loy - o.y) * inv.y, t2y = (hiy - o.y) * inv.y;
    float t1z = (loz - o.z) * inv.z, t2z = (hiz - o.z) * inv.z;
    float tmin = fmaxf(fmaxf(fminf(t1x, t2x), fmaxf(fminf(t1y, t2y), fminf(t1z, t2z))), tmin_ray);
    float tmax = fminf(fminf(fmaxf(t1x, t2x), fminf(fmaxf(t1y, t2y), fmaxf(t1z, t2z))), tmax_cur);
    *entry = tmin;
    return tmin <= tmax;
}

// moller_trumbore, crates/pyre/src/geometry/mesh.rs:153-178, without the
// final t-range test (the caller applies it).
__device__ __forceinline__ bool mt_test(const f3& o, const f3& d, const float4& A, const float4& B, const float4& C,
                                        float* t_out, float* u_out, float* v_out) {
    const f3 v0 = mk3(A.x, A.y, A.z), e1 = mk3(B.x, B.y, B.z), e2 = mk3(C.x, C.y, C.z);
    const f3 h = cross3(d, e2);
    const float a = dot3(e1, h);
    if (fabsf(a) < 1e-8f) return false;
    const float f = __frcp_rn(a);
    const f3 s = o - v0;
    const float u = f * dot3(s, h);
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    const f3 q = cross3(s, e1);
    const float v = f * dot3(d, q);
    if (v < 0.0f || u + v > 1.0f) return false;
    *t_out = f * dot3(e2, q);
    *u_out = u;
    *v_out = v;
    return true;
}

__device__ __forceinline__ f3 motion_offset(const DevInstance& I, float time) {
    // InstanceMotion::at (mesh.rs:53-55)
    return lerp3(mk3(I.off0[0], I.off0[1], I.off0[2]), mk3(I.off1[0], I.off1[1], I.off1[2]),
                 clampf_(time, 0.0f, 1.0f));
}

// Warp-synchronous two-level traversal (top-level BVH over instances, then
// each reached instance's BVH), equivalent to the instance scan of
// Scene::intersect / Scene::occluded (scene.rs:57-140): closest hit with the
// canonical tie rule, or any hit.
//
// trace_stream is a persistent loop for one warp over a queue of n rays: the
// lanes take rays from the queue through a shared work counter, and whenever
// at least `refill` lanes have finished their ray (or the warp has none), the
// idle lanes take new rays with one atomic for the warp, so the warp does not
// run on with a few long rays. A ray's traversal does not depend on which
// lane or warp runs it, so the results are the same as one ray per thread.
//
// Each lane keeps one tagged stack:
//   [0, 2^29)          node of an instance BVH
//   TOP | n            node of the top-level BVH
//   INST | slot        enter instance `slot` (root-box test, local origin)
//   INST | TOP | slot  enter static instance `slot`, whose root box the
//                      top-level step already tested
//   LEAF | n*W + k     leaf child k of wide node n (WIDTH > 2)
// A lane inside an instance leaves it (restores the world origin) when it
// reaches the next TOP or INST entry: those lie below the instance's nodes.
// With WIDTH 4 or 8 the instance BVHs are wide: a node step tests every
// child box, continues with the nearest hit child and pushes the others
// farthest first; leaf children are parked when they are reached.
// Inner nodes are stepped while more than 16 lanes of the warp still need a
// leaf (or no lane holds one); an any-hit lane that already holds one leaf
// keeps stepping speculatively, a closest-hit lane waits for the leaf phase
// (see STOP). Leaves found on the way are parked (at
// most three triangle ranges, all of the current instance: a lane holding
// leaves does not leave or enter an instance) and then tested by all lanes in
// lock step. An any-hit lane that finds a hit is finished at the end of that
// leaf phase.
//
// Src supplies the rays and takes the results (and kTmin / kTmax, the t range
// that idle lanes start with: the range of every ray where it is fixed):
//   uint32_t load(uint32_t j, TraceRay& r, int32_t& root)  ray j of the queue,
//            the top-level root to trace; returns the id passed to store
//   void store(uint32_t id, const TraceRay& r, TraceHit& h, bool found)
// All 32 lanes of the warp must call trace_stream with the same n and counter.
#define PYRE_TAG_LEAF (1 << 28)
#define PYRE_TAG_TOP (1 << 29)
#define PYRE_TAG_INST (1 << 30)
#define PYRE_NODE_NONE (-1)
// top-level leaves of one static instance are entered from the top-level
// step (INST|TOP entries); 0 keeps every instance behind an INST entry
#ifndef PYRE_TLAS_ENTER
#define PYRE_TLAS_ENTER 1
#endif

// Compare-exchange of (entry distance, stack entry) pairs, ascending.
__device__ __forceinline__ void cmp_swap(float& ea, int& na, float& eb, int& nb) {
    const bool sw = eb < ea;
    const float e = sw ? eb : ea;
    const int m = sw ? nb : na;
    eb = sw ? ea : eb;
    nb = sw ? na : nb;
    ea = e;
    na = m;
}
template <int W>
__device__ __forceinline__ void sort_children(float (&e)[W], int (&c)[W]) {
    if (W == 4) {  // optimal 5-comparator network
        cmp_swap(e[0], c[0], e[1], c[1]); cmp_swap(e[2], c[2], e[3], c[3]);
        cmp_swap(e[0], c[0], e[2], c[2]); cmp_swap(e[1], c[1], e[3], c[3]);
        cmp_swap(e[1], c[1], e[2], c[2]);
    } else {  // optimal 19-comparator network for 8
        constexpr int net[19][2] = {{0, 2}, {1, 3}, {4, 6}, {5, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}, {0, 1}, {2, 3},
                                    {4, 5}, {6, 7}, {2, 4}, {3, 5}, {1, 4}, {3, 6}, {1, 2}, {3, 4}, {5, 6}};
#pragma unroll
        for (int q = 0; q < 19; ++q) cmp_swap(e[net[q][0]], c[net[q][0]], e[net[q][1]], c[net[q][1]]);
    }
}

template <bool ANY, int WIDTH, class Src>
__device__ __forceinline__ void trace_stream(const DevScene& S, const Src& src, uint32_t n, uint32_t* counter,
                                             int refill) {
    // A lane stops stepping nodes once it holds STOP parked leaves (a binary
    // step can park two, a wide step at most one). A closest-hit lane stops
    // at its first: its leaves are then tested before its next node step, so
    // the boxes it culls with its current closest distance, and its hit, do
    // not depend on the other lanes of its warp. Where two triangles are hit
    // at distances a rounding apart, a box whose rounded entry lies between
    // them is culled or not depending on when the nearer hit was recorded;
    // with speculative steps that point moved with the warp, and about one
    // pixel in 10^6 of 1024^2 Cornell views changed from run to run. Any hit
    // culls with the ray's own fixed t_max, so its lanes keep stepping.
    constexpr int STOP = ANY ? (WIDTH > 2 ? 3 : 2) : 1;
    constexpr int LEAF_WAIT = ANY ? PYRE_LEAF_WAIT_ANY : PYRE_LEAF_WAIT_CLOSEST;
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lanes_below = (1u << lane) - 1u;
    bool drained = false;   // warp-uniform: the queue has no rays left
    bool active = false;    // the lane holds a ray
    uint32_t id = 0;
    TraceRay r;
    r.o = splat3(0.0f); r.d = mk3(0.0f, 0.0f, 1.0f); r.time = 0.0f; r.job = 0;
    r.tmin = Src::kTmin; r.tmax = Src::kTmax;  // a source whose rays share one range makes it a constant
    TraceHit hit;
    hit.inst = -1; hit.tri = -1; hit.light = -1; hit.t = 0.0f; hit.u = 0.0f; hit.v = 0.0f;
    f3 inv = splat3(0.0f);
    float best_t = 0.0f;
    bool found = false;
    bool hit_any = false;    // any-hit: the ray is occluded
    bool exhausted = true;   // no node left to step
    // an 8-wide step can push 7 entries, so the 8-wide stack is deeper
    constexpr int STACK = WIDTH == 8 ? 96 : PYRE_STACK;
    // Any-hit traversal keeps the bottom 8 stack entries of each lane in
    // shared memory (entry-major, so a lane always uses its own bank), the
    // rest in local memory: the shadow stage is 4 % faster on the 1080p frame
    // (4 or 12 entries are slower than 8).
    // Closest hit keeps the whole stack in local memory; with the same short
    // stack it was 0.6 % slower (4 entries), 2 % (8) and 4 % (16).
    constexpr int SK = ANY ? 8 : 0;
    __shared__ int sstack[SK > 0 ? SK : 1][128];  // traversal blocks have at most 128 threads
    int stack[STACK - SK];
    int sp = 0;
    auto spush = [&](int v) {
        if (SK > 0 && sp < SK) sstack[sp][threadIdx.x] = v;
        else stack[sp - SK] = v;
        ++sp;
    };
    auto spop = [&]() -> int {
        --sp;
        return (SK > 0 && sp < SK) ? sstack[sp][threadIdx.x] : stack[sp - SK];
    };
    int node = PYRE_NODE_NONE;
    int inst = -1;
    f3 o = r.o;
    // Parked triangle ranges: an any-hit lane keeps stepping (speculatively)
    // while it holds at most one, so one node step never needs more than
    // three; a closest-hit lane parks at most the two leaves of one binary
    // step, and keeps two: fewer spills at the kernel's 56 registers (28
    // against 34 B stored), 803.0 against 792.9 Msamples/s on the 1080p
    // studio frame (extend 89.6 against 91.7 ms)
    constexpr int PR = ANY ? 3 : 2;
    int ls[PR], lc[PR];
#pragma unroll
    for (int q = 0; q < PR; ++q) { ls[q] = 0; lc[q] = 0; }
    int parked = 0;

    while (true) {
        // ---- refill idle lanes from the queue
        if (!drained) {
            const unsigned idle = __ballot_sync(FULL, !active);
            const int n_idle = __popc(idle);
            if (n_idle >= refill || n_idle == 32) {
                const int leader = __ffs(idle) - 1;
                uint32_t base = 0;
                if (lane == leader) base = atomicAdd(counter, (uint32_t)n_idle);
                base = __shfl_sync(FULL, base, leader);
                if ((uint64_t)base + (uint64_t)n_idle >= (uint64_t)n) drained = true;
                const uint32_t j = base + (uint32_t)__popc(idle & lanes_below);
                if (!active && j < n) {
                    int32_t root;
                    id = src.load(j, r, root);
                    active = true;
                    inv = mk3(__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z));
                    hit.inst = -1; hit.tri = -1;
                    hit.u = 0.0f; hit.v = 0.0f;
                    best_t = r.tmax;
                    found = false;
                    hit_any = false;
                    exhausted = root < 0;
                    sp = 0;
                    node = exhausted ? PYRE_NODE_NONE : (root | PYRE_TAG_TOP);
                    inst = -1;
                    o = r.o;
                    parked = 0;
#pragma unroll
                    for (int q = 0; q < PR; ++q) lc[q] = 0;
                }
            }
        }
        if (!__any_sync(FULL, active)) {
            if (drained) break;
            continue;
        }
        // ---- inner phase: step nodes until at most LEAF_WAIT lanes still
        // look for a leaf. Those lanes sit out the leaf phase and resume after
        // it; the others do not idle until the slowest lane reaches its first
        // leaf. The phase also runs while no lane holds a leaf to test, so each
        // round makes progress.
        while (true) {
            const int seeking = __popc(__ballot_sync(FULL, active && !exhausted && !hit_any && parked == 0));
            if (seeking == 0) break;
            if (seeking <= LEAF_WAIT && __any_sync(FULL, active && !hit_any && parked > 0)) break;
            // each lane takes up to PYRE_STEPS_PER_VOTE node steps between the warp's votes
#pragma unroll 1
            for (int step = 0; step < PYRE_STEPS_PER_VOTE; ++step) {
                if (!active || exhausted || hit_any || parked >= STOP) break;
                if (node == PYRE_NODE_NONE) {
                    if (sp == 0) { exhausted = true; continue; }
                    node = spop();
                }
                // a top-level entry reached inside an instance: the instance's
                // BVH is done, so the lane leaves it (once its parked leaves,
                // which belong to the instance, are tested). Leaving without a
                // stack entry of its own saves a node step per instance:
                // 710.2 against 703.7 Msamples/s on the 1080p studio frame,
                // closest hit 4.04 against 4.34 ms on the microbenchmark.
                // Tag bits are tested once per step, and instance BVH nodes
                // (two thirds of the steps) skip the rest: 770.9 against
                // 767.4 Msamples/s on the 1080p studio frame. A closest-hit
                // lane that steps holds no parked leaf (STOP is 1).
                if (node & (PYRE_TAG_TOP | PYRE_TAG_INST)) {  // a top-level node or an instance entry
                    if (inst >= 0) {
                        if (ANY && parked) { spush(node); node = PYRE_NODE_NONE; parked = STOP; continue; }
                        inst = -1;
                        o = r.o;
                    }
                    if ((node & (PYRE_TAG_INST | PYRE_TAG_TOP)) == (PYRE_TAG_INST | PYRE_TAG_TOP)) {
                        // a static instance whose root box the top-level step
                        // tested: enter it and step its root node in this step
                        // (the lane is at the top level, so o is the world origin)
                        const int k = node & ~(PYRE_TAG_INST | PYRE_TAG_TOP);
                        node = WIDTH > 2 ? __ldg(S.wroot + k) : __ldg(&S.inst[k].blas_root);
                        if (node < 0) { node = PYRE_NODE_NONE; continue; }
                        inst = k;
                    } else if (node & PYRE_TAG_INST) {
                        if (ANY && parked) { spush(node); node = PYRE_NODE_NONE; parked = STOP; continue; }
                        const int k = node & ~PYRE_TAG_INST;
                        node = PYRE_NODE_NONE;
                        const DevInstance& I = S.inst[k];
                        const int root = WIDTH > 2 ? S.wroot[k] : I.blas_root;
                        if (root < 0) continue;
                        f3 lo = r.o;
                        if (I.has_motion) {
                            f3 off = motion_offset(I, r.time);
                            if (!is_zero3(off)) lo = r.o - off;
                        }
                        float e;
                        if (!slab(I.lo[0], I.hi[0], I.lo[1], I.hi[1], I.lo[2], I.hi[2], lo, inv, r.tmin, best_t, &e))
                            continue;
                        inst = k;
                        o = lo;
                        node = root;
                        continue;
                    }
                }
                const bool top = (node & PYRE_TAG_TOP) != 0;
                if (WIDTH > 2 && !top) {
                    if (node & PYRE_TAG_LEAF) {  // park a leaf child of a wide node
                        const uint32_t ref = (uint32_t)(node & ~PYRE_TAG_LEAF);
                        const int32_t* NI = reinterpret_cast<const int32_t*>(S.wnodes) +
                                            (size_t)(ref / WIDTH) * (PYRE_WIDE_FIELDS * WIDTH) + ref % WIDTH;
                        ls[parked] = __ldg(NI + 6 * WIDTH);
                        lc[parked] = __ldg(NI + 7 * WIDTH);
                        ++parked;
                        node = PYRE_NODE_NONE;
                        continue;
                    }
                    constexpr int Q = WIDTH / 4;  // float4 rows per field
                    const float4* N = S.wnodes + (size_t)node * (2 * WIDTH);
                    float e[WIDTH];
                    int ent[WIDTH];
    #pragma unroll
                    for (int q = 0; q < Q; ++q) {
                        const float4 lx = __ldg(N + 0 * Q + q), hx = __ldg(N + 1 * Q + q), ly = __ldg(N + 2 * Q + q),
                                     hy = __ldg(N + 3 * Q + q), lz = __ldg(N + 4 * Q + q), hz = __ldg(N + 5 * Q + q);
                        const int4 ch = __ldg(reinterpret_cast<const int4*>(N + 6 * Q + q));
                        const int4 ct = __ldg(reinterpret_cast<const int4*>(N + 7 * Q + q));
                        const float LX[4] = {lx.x, lx.y, lx.z, lx.w}, HX[4] = {hx.x, hx.y, hx.z, hx.w};
                        const float LY[4] = {ly.x, ly.y, ly.z, ly.w}, HY[4] = {hy.x, hy.y, hy.z, hy.w};
                        const float LZ[4] = {lz.x, lz.y, lz.z, lz.w}, HZ[4] = {hz.x, hz.y, hz.z, hz.w};
                        const int CH[4] = {ch.x, ch.y, ch.z, ch.w}, CT[4] = {ct.x, ct.y, ct.z, ct.w};
    #pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            float ek;
                            const bool h = CH[k] >= 0 && slab(LX[k], HX[k], LY[k], HY[k], LZ[k], HZ[k], o, inv, r.tmin,
                                                              best_t, &ek);
                            e[4 * q + k] = h ? ek : __int_as_float(0x7f800000);
                            ent[4 * q + k] = !h ? PYRE_NODE_NONE
                                                : (CT[k] > 0 ? (PYRE_TAG_LEAF | (node * WIDTH + 4 * q + k)) : CH[k]);
                        }
                    }
                    sort_children<WIDTH>(e, ent);
                    int nh = 0;
    #pragma unroll
                    for (int k = 1; k < WIDTH; ++k) nh += ent[k] != PYRE_NODE_NONE ? 1 : 0;
                    if (sp + nh > STACK) { atomicExch(S.error_flag, -5); exhausted = true; sp = 0; continue; }
    #pragma unroll
                    for (int k = WIDTH - 1; k >= 1; --k)
                        if (ent[k] != PYRE_NODE_NONE) spush(ent[k]);
                    node = ent[0];
                    continue;
                }
                const float4* N = S.nodes + 4 * (size_t)(node & ~PYRE_TAG_TOP);
#if PYRE_LD256
                float4 na, nb, nc, ndf;
                ldg_256(N, na, nb);
                ldg_256(N + 2, nc, ndf);
                const int4 nd = make_int4(__float_as_int(ndf.x), __float_as_int(ndf.y), __float_as_int(ndf.z),
                                          __float_as_int(ndf.w));
#else
                const float4 na = __ldg(N), nb = __ldg(N + 1), nc = __ldg(N + 2);
                const int4 nd = __ldg(reinterpret_cast<const int4*>(N + 3));
#endif
                float e0, e1;
                const bool h0 = nd.x >= 0 && slab(na.x, na.y, na.z, na.w, nc.x, nc.y, o, inv, r.tmin, best_t, &e0);
                const bool h1 = nd.y >= 0 && slab(nb.x, nb.y, nb.z, nb.w, nc.z, nc.w, o, inv, r.tmin, best_t, &e1);
                node = PYRE_NODE_NONE;
                const bool leaf0 = nd.z > 0, leaf1 = nd.w > 0;
                // leaves: park triangle ranges, or queue the instances of a top-level leaf
                if (top) {
                    const int need = (h0 && leaf0 ? nd.z : 0) + (h1 && leaf1 ? nd.w : 0) + 1;
                    if (sp + need > STACK) { atomicExch(S.error_flag, -5); exhausted = true; sp = 0; continue; }
                    if (h1 && leaf1)
                        for (int k = nd.w - 1; k >= 0; --k) spush(PYRE_TAG_INST | (nd.y + k));
                    if (h0 && leaf0)
                        for (int k = nd.z - 1; k >= 0; --k) spush(PYRE_TAG_INST | (nd.x + k));
                } else {
                    if (h0 && leaf0) { ls[parked] = nd.x; lc[parked] = nd.z; ++parked; }
                    if (h1 && leaf1) { ls[parked] = nd.y; lc[parked] = nd.w; ++parked; }
                }
                const int tag = top ? PYRE_TAG_TOP : 0;
                const bool g0 = h0 && !leaf0, g1 = h1 && !leaf1;
                if (g0 && g1) {
                    const bool first0 = e0 <= e1;
                    if (sp >= STACK) { atomicExch(S.error_flag, -5); exhausted = true; sp = 0; continue; }
                    spush((first0 ? nd.y : nd.x) | tag);
                    node = (first0 ? nd.x : nd.y) | tag;
                } else if (g0) {
                    node = nd.x | tag;
                } else if (g1) {
                    node = nd.y | tag;
                }
            }
        }
        // ---- leaf phase: all lanes test their parked triangles together
        const bool testing = active && !hit_any;
        const int c0 = testing ? lc[0] : 0, c1 = testing ? lc[1] : 0, c2 = (PR > 2 && testing) ? lc[PR - 1] : 0;
        const int total = parked == 0 ? 0 : c0 + (parked > 1 ? c1 : 0) + (PR > 2 && parked > 2 ? c2 : 0);
        const int kmax = __reduce_max_sync(FULL, total);
        for (int k = 0; k < kmax; ++k) {
            if (k >= total || hit_any) continue;
            const int slot = k < c0 ? ls[0] + k : (k < c0 + c1 ? ls[1] + (k - c0) : ls[PR - 1] + (k - c0 - c1));
            const float4 A = __ldg(S.tris + 3 * (size_t)slot), B = __ldg(S.tris + 3 * (size_t)slot + 1),
                         C = __ldg(S.tris + 3 * (size_t)slot + 2);
            float t, u, v;
            if (!mt_test(o, r.d, A, B, C, &t, &u, &v)) continue;
            if (!(t > r.tmin && t < r.tmax)) continue;
            if (ANY) { found = true; hit_any = true; continue; }
            bool better = t < best_t;
            if (!better && t == best_t && found) {
                // a tie (rare): the lower Scene::primitives index, then the lower
                // triangle id, wins; both are read back from the records
                const int32_t cur = S.inst[inst].orig_id, best = S.inst[hit.inst].orig_id;
                const uint32_t key = __float_as_uint(A.w);
                const uint32_t best_key = __float_as_uint(__ldg(S.tris + 3 * (size_t)hit.tri).w);
                better = cur < best || (cur == best && key < best_key);
            }
            if (better) {
                best_t = t;
                found = true;
                hit.u = u; hit.v = v;
                hit.inst = inst; hit.tri = slot;
            }
        }
        parked = 0;
#pragma unroll
        for (int q = 0; q < PR; ++q) lc[q] = 0;
        // ---- finished rays hand over their result; the lane becomes idle
        if (active && (exhausted || hit_any)) {
            hit.t = best_t;
            hit.light = -1;
            src.store(id, r, hit, found);
            active = false;
        }
    }
}

// DiffuseAreaQuadLight::intersect_plane (light.rs:86-107).
__device__ __forceinline__ bool quad_intersect(const DevQuadLight& L, const f3& o, const f3& d, float tmin, float tmax,
                                               float* t_out, f3* p_out) {
    float denom = dot3(d, L.normal);
    if (fabsf(denom) < 1e-9f) return false;
    float t = dot3(L.p0 - o, L.normal) / denom;
    if (t < tmin || t > tmax) return false;
    f3 p = o + t * d;
    f3 dd = p - L.p0;
    float alpha = dot3(cross3(dd, L.edge_v), L.crs) * L.inv_cross_len_sq;
    if (!(alpha >= 0.0f && alpha <= 1.0f)) return false;
    float beta = dot3(cross3(L.edge_u, dd), L.crs) * L.inv_cross_len_sq;
    if (!(beta >= 0.0f && beta <= 1.0f)) return false;
    *t_out = t;
    *p_out = p;
    return true;
}

// Quad lights after primitives with strict `<` (scene.rs:78-94): lights
// [light_first, light_first + light_count) can replace the closest hit.
__device__ __forceinline__ void hit_quad_lights(const DevScene& S, const TraceRay& r, uint32_t light_first,
                                                uint32_t light_count, TraceHit* hit) {
    float best = hit->inst >= 0 ? hit->t : r.tmax;
    for (uint32_t l = light_first; l < light_first + light_count; ++l) {
        float t; f3 p;
        if (quad_intersect(S.lights[l], r.o, r.d, r.tmin, best, &t, &p) && t < best) {
            best = t;
            hit->t = t; hit->light = (int32_t)l;
        }
    }
}

}  // namespace pyre
