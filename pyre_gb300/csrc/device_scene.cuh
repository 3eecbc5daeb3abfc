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
//   normal float[3*V]   vertex normals (meshes without normals use e1 x e2)
#pragma once
#include <cuda_runtime.h>
#include "pyre_math.cuh"

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
    const DevMaterial* materials;
    uint32_t n_materials;
    const DevQuadLight* lights;
    uint32_t n_lights;
    int has_env;
    DevEnv env;
    int* error_flag;       // set to PYRE_ERR_OVERFLOW by a kernel that hit a limit
};

struct TraceRay {
    f3 o, d;
    float tmin, tmax, time;
};

struct TraceHit {
    float t, u, v;
    int32_t inst;  // instance slot (device order); -1 = no hit
    int32_t tri;   // triangle slot
    int32_t light; // quad light index when the closest hit is a light, else -1
};

#define PYRE_STACK 64

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

// Traverses one instance's BVH. Closest: tightens *best_t and records the hit
// with the canonical tie rule. Any: returns true on the first admissible hit.
template <bool ANY>
__device__ __forceinline__ bool trace_blas(const DevScene& S, const DevInstance& I, int32_t islot, const TraceRay& r,
                                           const f3& inv, float* best_t, TraceHit* hit, uint32_t* best_key_tri,
                                           int* stack) {
    f3 o = r.o;
    if (I.has_motion) {
        f3 off = motion_offset(I, r.time);
        if (!is_zero3(off)) o = r.o - off;
    }
    float entry;
    if (!slab(I.lo[0], I.hi[0], I.lo[1], I.hi[1], I.lo[2], I.hi[2], o, inv, r.tmin, *best_t, &entry)) return false;
    int sp = 0;
    int node = I.blas_root;
    while (true) {
        const float4* N = S.nodes + 4 * (size_t)node;
        const float4 na = __ldg(N), nb = __ldg(N + 1), nc = __ldg(N + 2);
        const int4 nd = __ldg(reinterpret_cast<const int4*>(N + 3));
        float e0, e1;
        bool h0 = nd.x >= 0 && slab(na.x, na.y, na.z, na.w, nc.x, nc.y, o, inv, r.tmin, *best_t, &e0);
        bool h1 = nd.y >= 0 && slab(nb.x, nb.y, nb.z, nb.w, nc.z, nc.w, o, inv, r.tmin, *best_t, &e1);
        // Leaves are tested in place; interior children are followed.
        int kids[2] = {nd.x, nd.y};
        int counts[2] = {nd.z, nd.w};
        bool go[2] = {false, false};
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            bool hc = c == 0 ? h0 : h1;
            if (!hc) continue;
            if (counts[c] > 0) {
                for (int k = kids[c]; k < kids[c] + counts[c]; ++k) {
                    const float4 A = __ldg(S.tris + 3 * (size_t)k), B = __ldg(S.tris + 3 * (size_t)k + 1),
                                 C = __ldg(S.tris + 3 * (size_t)k + 2);
                    float t, u, v;
                    if (!mt_test(o, r.d, A, B, C, &t, &u, &v)) continue;
                    if (!(t > r.tmin && t < r.tmax)) continue;
                    if (ANY) return true;
                    const uint32_t key = __float_as_uint(A.w);
                    bool better = t < *best_t;
                    if (!better && t == *best_t && hit->inst >= 0) {
                        const int32_t oi = I.orig_id, ob = S.inst[hit->inst].orig_id;
                        better = oi < ob || (oi == ob && key < *best_key_tri);
                    }
                    if (better) {
                        *best_t = t;
                        hit->t = t; hit->u = u; hit->v = v;
                        hit->inst = islot; hit->tri = k;
                        *best_key_tri = key;
                    }
                }
            } else {
                go[c] = true;
            }
        }
        if (go[0] && go[1]) {
            // nearer child next, farther one on the stack
            int nearc = e0 <= e1 ? kids[0] : kids[1];
            int farc = e0 <= e1 ? kids[1] : kids[0];
            if (sp >= PYRE_STACK) { atomicExch(S.error_flag, -5); return false; }
            stack[sp++] = farc;
            node = nearc;
        } else if (go[0]) {
            node = kids[0];
        } else if (go[1]) {
            node = kids[1];
        } else {
            if (sp == 0) break;
            node = stack[--sp];
        }
    }
    return false;
}

// Scene traversal: the top-level BVH over instance swept bounds, then each
// reached instance's BVH. Equivalent to the instance scan of Scene::intersect
// / Scene::occluded (scene.rs:57-140) for closest (with the canonical tie
// rule) and any hit.
template <bool ANY>
__device__ bool trace_scene(const DevScene& S, const TraceRay& r, TraceHit* hit) {
    hit->inst = -1; hit->tri = -1; hit->light = -1;
    hit->t = r.tmax; hit->u = 0.0f; hit->v = 0.0f;
    float best_t = r.tmax;
    uint32_t best_key = 0xffffffffu;
    const f3 inv = mk3(__frcp_rn(r.d.x), __frcp_rn(r.d.y), __frcp_rn(r.d.z));
    int stack[PYRE_STACK];
    if (S.tlas_root >= 0) {
        int tstack[PYRE_STACK];
        int tsp = 0;
        int node = S.tlas_root;
        while (true) {
            const float4* N = S.nodes + 4 * (size_t)node;
            const float4 na = __ldg(N), nb = __ldg(N + 1), nc = __ldg(N + 2);
            const int4 nd = __ldg(reinterpret_cast<const int4*>(N + 3));
            float e0, e1;
            bool h0 = nd.x >= 0 && slab(na.x, na.y, na.z, na.w, nc.x, nc.y, r.o, inv, r.tmin, best_t, &e0);
            bool h1 = nd.y >= 0 && slab(nb.x, nb.y, nb.z, nb.w, nc.z, nc.w, r.o, inv, r.tmin, best_t, &e1);
            int kids[2] = {nd.x, nd.y};
            int counts[2] = {nd.z, nd.w};
            bool go[2] = {false, false};
            for (int c = 0; c < 2; ++c) {
                bool hc = c == 0 ? h0 : h1;
                if (!hc) continue;
                if (counts[c] > 0) {
                    for (int k = kids[c]; k < kids[c] + counts[c]; ++k) {
                        const DevInstance I = S.inst[k];
                        if (I.blas_root < 0) continue;
                        if (trace_blas<ANY>(S, I, k, r, inv, &best_t, hit, &best_key, stack)) return true;
                    }
                } else {
                    go[c] = true;
                }
            }
            if (go[0] && go[1]) {
                int nearc = e0 <= e1 ? kids[0] : kids[1];
                int farc = e0 <= e1 ? kids[1] : kids[0];
                if (tsp >= PYRE_STACK) { atomicExch(S.error_flag, -5); break; }
                tstack[tsp++] = farc;
                node = nearc;
            } else if (go[0]) {
                node = kids[0];
            } else if (go[1]) {
                node = kids[1];
            } else {
                if (tsp == 0) break;
                node = tstack[--tsp];
            }
        }
    }
    if (ANY) return false;
    return hit->inst >= 0;
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

// Closest hit including quad lights (lights after primitives with strict `<`,
// scene.rs:78-94).
__device__ __forceinline__ void trace_closest_with_lights(const DevScene& S, const TraceRay& r, TraceHit* hit) {
    trace_scene<false>(S, r, hit);
    float best = hit->inst >= 0 ? hit->t : r.tmax;
    for (uint32_t l = 0; l < S.n_lights; ++l) {
        float t; f3 p;
        if (quad_intersect(S.lights[l], r.o, r.d, r.tmin, best, &t, &p) && t < best) {
            best = t;
            hit->t = t; hit->light = (int32_t)l;
        }
    }
}

}  // namespace pyre
