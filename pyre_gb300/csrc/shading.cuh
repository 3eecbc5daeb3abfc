// shading.cuh — BSDFs, lights, environment and camera on the device.
//
// Each function restates the Pyre CPU function cited beside it with the same
// binary32 operation order (translation units are built with --fmad=false).
// Transcendentals use CUDA's full-precision sinf/cosf/acosf/atan2f, which can
// differ from glibc by an ulp; images are therefore compared statistically.
#pragma once
#include "../../include/pyre_cuda.h"
#include "device_scene.cuh"

namespace pyre {

// ---------------------------------------------------------------- frame ----
struct Frame3 {  // math.rs:88-104
    f3 t, bt, n;
};
__device__ __forceinline__ Frame3 frame_from_normal(f3 n) {
    f3 helper = fabsf(n.x) > 0.9f ? mk3(0.0f, 1.0f, 0.0f) : mk3(1.0f, 0.0f, 0.0f);
    Frame3 f;
    f.t = normalize3(cross3(helper, n));
    f.bt = cross3(n, f.t);
    f.n = n;
    return f;
}
__device__ __forceinline__ f3 to_local(const Frame3& f, f3 v) { return mk3(dot3(v, f.t), dot3(v, f.bt), dot3(v, f.n)); }
__device__ __forceinline__ f3 to_world(const Frame3& f, f3 v) { return v.x * f.t + v.y * f.bt + v.z * f.n; }

__device__ __forceinline__ float power_heuristic(float pa, float pb) {  // integrator.rs:234-240
    float a2 = pa * pa, b2 = pb * pb, denom = a2 + b2;
    return denom > 0.0f ? a2 / denom : 0.0f;
}

// ---------------------------------------------------------------- BSDFs ----
__device__ __forceinline__ float luminance(f3 c) { return dot3(c, mk3(0.2126f, 0.7152f, 0.0722f)); }
__device__ __forceinline__ f3 cosine_sample_hemisphere(f2 u) {  // material.rs:239-246
    float r = sqrtf(u.x);
    float phi = 2.0f * PYRE_PI * u.y;
    float s, c;
    sincosf(phi, &s, &c);
    return mk3(r * c, r * s, sqrtf(fmaxf(1.0f - u.x, 0.0f)));
}
__device__ __forceinline__ float ggx_d(f3 h, float alpha) {  // material.rs:249-256
    if (h.z <= 0.0f) return 0.0f;
    float a2 = alpha * alpha;
    float denom = h.z * h.z * (a2 - 1.0f) + 1.0f;
    return a2 / (PYRE_PI * denom * denom);
}
__device__ __forceinline__ f3 schlick(float cos_d, f3 f0) {  // material.rs:259-262
    float c = clampf_(cos_d, 0.0f, 1.0f);
    return f0 + (splat3(1.0f) - f0) * powi5(1.0f - c);
}
__device__ __forceinline__ float ggx_lambda(f3 v, float alpha) {  // material.rs:264-272
    float cos2 = v.z * v.z;
    if (cos2 >= 1.0f) return 0.0f;
    float a2 = alpha * alpha;
    float tan2 = (1.0f - cos2) / fmaxf(cos2, 1e-8f);
    return 0.5f * (-1.0f + sqrtf(1.0f + a2 * tan2));
}

struct Bsdf {
    uint32_t kind;
    f3 base;
    float metallic, roughness, specular;
};
__device__ __forceinline__ Bsdf load_bsdf(const DevScene& S, uint32_t m) {
    const DevMaterial M = S.materials[m];
    Bsdf b;
    b.kind = M.kind;
    b.base = mk3(M.base[0], M.base[1], M.base[2]);
    b.metallic = M.metallic; b.roughness = M.roughness; b.specular = M.specular;
    return b;
}
__device__ __forceinline__ float bsdf_alpha(const Bsdf& b) { return fmaxf(b.roughness * b.roughness, 1e-3f); }
__device__ __forceinline__ f3 bsdf_f0(const Bsdf& b) { return lerp3(splat3(0.08f * b.specular), b.base, b.metallic); }
__device__ __forceinline__ void lobe_weights(const Bsdf& b, float* pd, float* ps) {  // material.rs:112-121
    float diff = (1.0f - b.metallic) * luminance(b.base);
    float spec = fmaxf(luminance(bsdf_f0(b)), 0.04f);
    float total = diff + spec;
    if (total > 0.0f) { *pd = diff / total; *ps = spec / total; }
    else { *pd = 1.0f; *ps = 0.0f; }
}

__device__ __forceinline__ f3 bsdf_eval(const Bsdf& b, f3 wo, f3 wi) {
    if (b.kind == PYRE_MAT_LAMBERTIAN) {  // material.rs:52-58
        if (wo.z <= 0.0f || wi.z <= 0.0f) return splat3(0.0f);
        return b.base / PYRE_PI;
    }
    f3 fd = splat3(0.0f), fs = splat3(0.0f);
    // eval_diffuse, material.rs:125-138
    if (!(wo.z <= 0.0f || wi.z <= 0.0f || b.metallic >= 1.0f)) {
        f3 h = normalize_or_zero3(wo + wi);
        if (!(len2(h) < 1e-10f)) {
            float cos_d = clampf_(dot3(wi, h), 0.0f, 1.0f);
            float fd90 = 0.5f + 2.0f * b.roughness * cos_d * cos_d;
            float fd_v = 1.0f + (fd90 - 1.0f) * powi5(fmaxf(1.0f - wo.z, 0.0f));
            float fd_l = 1.0f + (fd90 - 1.0f) * powi5(fmaxf(1.0f - wi.z, 0.0f));
            fd = b.base * (1.0f - b.metallic) / PYRE_PI * fd_v * fd_l;
        }
    }
    // eval_specular, material.rs:142-155
    if (!(wo.z <= 0.0f || wi.z <= 0.0f)) {
        f3 h = normalize_or_zero3(wo + wi);
        if (!(len2(h) < 1e-10f || h.z <= 0.0f)) {
            float a = bsdf_alpha(b);
            float d = ggx_d(h, a);
            f3 f = schlick(fmaxf(dot3(wi, h), 0.0f), bsdf_f0(b));
            float g = 1.0f / (1.0f + ggx_lambda(wo, a) + ggx_lambda(wi, a));
            fs = d * f * g / (4.0f * wo.z * wi.z);
        }
    }
    return fd + fs;
}

__device__ __forceinline__ float bsdf_pdf(const Bsdf& b, f3 wo, f3 wi) {
    if (b.kind == PYRE_MAT_LAMBERTIAN) {  // material.rs:60-66
        if (wo.z <= 0.0f || wi.z <= 0.0f) return 0.0f;
        return wi.z / PYRE_PI;
    }
    float pd, ps;
    lobe_weights(b, &pd, &ps);
    float pdf_d = wi.z <= 0.0f ? 0.0f : wi.z / PYRE_PI;  // material.rs:157-163
    float pdf_s = 0.0f;                                 // material.rs:168-180
    if (!(wo.z <= 0.0f || wi.z <= 0.0f)) {
        f3 h = normalize_or_zero3(wo + wi);
        if (!(len2(h) < 1e-10f || h.z <= 0.0f)) {
            float a = bsdf_alpha(b);
            float d = ggx_d(h, a);
            float g1 = 1.0f / (1.0f + ggx_lambda(wo, a));
            pdf_s = g1 * d / (4.0f * wo.z);
        }
    }
    return pd * pdf_d + ps * pdf_s;
}

// bsdf_eval and bsdf_pdf of the same (wo, wi) in one pass: the half vector,
// the GGX D term and Lambda(wo) are computed once and shared. Each output
// goes through the same binary32 operations, in the same order, as the two
// functions above, so it is bit-identical to them.
__device__ __forceinline__ void bsdf_eval_pdf(const Bsdf& b, f3 wo, f3 wi, f3* f_out, float* pdf_out) {
    const bool upper = !(wo.z <= 0.0f || wi.z <= 0.0f);
    if (b.kind == PYRE_MAT_LAMBERTIAN) {
        *f_out = upper ? b.base / PYRE_PI : splat3(0.0f);
        *pdf_out = upper ? wi.z / PYRE_PI : 0.0f;
        return;
    }
    f3 fd = splat3(0.0f), fs = splat3(0.0f);
    float pdf_s = 0.0f;
    if (upper) {
        const f3 h = normalize_or_zero3(wo + wi);
        if (!(len2(h) < 1e-10f)) {
            if (!(b.metallic >= 1.0f)) {  // eval_diffuse
                float cos_d = clampf_(dot3(wi, h), 0.0f, 1.0f);
                float fd90 = 0.5f + 2.0f * b.roughness * cos_d * cos_d;
                float fd_v = 1.0f + (fd90 - 1.0f) * powi5(fmaxf(1.0f - wo.z, 0.0f));
                float fd_l = 1.0f + (fd90 - 1.0f) * powi5(fmaxf(1.0f - wi.z, 0.0f));
                fd = b.base * (1.0f - b.metallic) / PYRE_PI * fd_v * fd_l;
            }
            if (!(h.z <= 0.0f)) {  // eval_specular and pdf_specular
                const float a = bsdf_alpha(b);
                const float d = ggx_d(h, a);
                const float one_lo = 1.0f + ggx_lambda(wo, a);
                const f3 f = schlick(fmaxf(dot3(wi, h), 0.0f), bsdf_f0(b));
                const float g = 1.0f / (one_lo + ggx_lambda(wi, a));
                fs = d * f * g / (4.0f * wo.z * wi.z);
                const float g1 = 1.0f / one_lo;
                pdf_s = g1 * d / (4.0f * wo.z);
            }
        }
    }
    *f_out = fd + fs;
    float pd, ps;
    lobe_weights(b, &pd, &ps);
    const float pdf_d = wi.z <= 0.0f ? 0.0f : wi.z / PYRE_PI;
    *pdf_out = pd * pdf_d + ps * pdf_s;
}

__device__ __forceinline__ f3 sample_ggx_vndf(f3 wo, float alpha, f2 u) {  // material.rs:291-317
    f3 vh = normalize3(mk3(alpha * wo.x, alpha * wo.y, wo.z));
    float lensq = vh.x * vh.x + vh.y * vh.y;
    f3 t1 = lensq > 0.0f ? mk3(-vh.y, vh.x, 0.0f) / sqrtf(lensq) : mk3(1.0f, 0.0f, 0.0f);
    f3 t2 = cross3(vh, t1);
    float r = sqrtf(u.x);
    float phi = 2.0f * PYRE_PI * u.y;
    float sp, cp;
    sincosf(phi, &sp, &cp);
    float t1c = r * cp;
    float t2c = r * sp;
    float s = 0.5f * (1.0f + vh.z);
    t2c = (1.0f - s) * sqrtf(fmaxf(1.0f - t1c * t1c, 0.0f)) + s * t2c;
    f3 nh = t1c * t1 + t2c * t2 + sqrtf(fmaxf(1.0f - t1c * t1c - t2c * t2c, 0.0f)) * vh;
    return normalize3(mk3(alpha * nh.x, alpha * nh.y, fmaxf(nh.z, 0.0f)));
}

// The direction drawn by Bsdf::sample (material.rs:68-76 Lambertian,
// 197-222 Disney); false where the reference returns None before it
// evaluates the pdf. A Lambertian draw always has wi.z > 0 (u.x < 1).
__device__ __forceinline__ bool bsdf_sample_dir(const Bsdf& b, f3 wo, f2 u, f3* wi_out) {
    if (wo.z <= 0.0f) return false;
    if (b.kind == PYRE_MAT_LAMBERTIAN) {
        *wi_out = cosine_sample_hemisphere(u);
        return true;
    }
    float pd, ps;
    lobe_weights(b, &pd, &ps);
    if (pd + ps <= 0.0f) return false;
    f3 wi;
    if (u.x < pd) {
        f2 ur; ur.x = fminf(u.x / pd, 1.0f - 1e-7f); ur.y = u.y;
        wi = cosine_sample_hemisphere(ur);
    } else {
        f2 ur; ur.x = fminf((u.x - pd) / ps, 1.0f - 1e-7f); ur.y = u.y;
        f3 h = sample_ggx_vndf(wo, bsdf_alpha(b), ur);
        wi = 2.0f * dot3(wo, h) * h - wo;  // reflect, material.rs:285-287
    }
    if (wi.z <= 0.0f) return false;
    *wi_out = wi;
    return true;
}

// Bsdf::sample (material.rs:68-76, 197-225): the drawn direction with
// eval and pdf there; None where the pdf is not positive (Disney).
__device__ __forceinline__ bool bsdf_sample(const Bsdf& b, f3 wo, f2 u, f3* wi_out, f3* f_out, float* pdf_out) {
    f3 wi;
    if (!bsdf_sample_dir(b, wo, u, &wi)) return false;
    f3 f;
    float p;
    bsdf_eval_pdf(b, wo, wi, &f, &p);
    if (b.kind != PYRE_MAT_LAMBERTIAN && p <= 0.0f) return false;
    *wi_out = wi;
    *f_out = f;
    *pdf_out = p;
    return true;
}

// ---------------------------------------------------------- quad lights ----
// DiffuseAreaQuadLight::sample, light.rs:111-133
__device__ __forceinline__ bool quad_sample(const DevQuadLight& L, f3 from, f2 u, f3* pos, f3* wi_out, float* pdf) {
    f3 p = L.p0 + u.x * L.edge_u + u.y * L.edge_v;
    f3 to_light = p - from;
    float dist2 = len2(to_light);
    if (dist2 <= 0.0f) return false;
    float dist = sqrtf(dist2);
    f3 wi = to_light / dist;
    float cos_light = -dot3(wi, L.normal);
    if (cos_light <= 0.0f) return false;
    *pdf = dist2 / (cos_light * L.area);
    *pos = p;
    *wi_out = wi;
    return true;
}
// DiffuseAreaQuadLight::pdf, light.rs:135-144
__device__ __forceinline__ float quad_pdf(const DevQuadLight& L, f3 from, f3 wi) {
    float t; f3 p;
    if (!quad_intersect(L, from, wi, 1e-4f, __int_as_float(0x7f800000), &t, &p)) return 0.0f;
    float cos_light = -dot3(wi, L.normal);
    if (cos_light <= 0.0f) return 0.0f;
    return t * t / (cos_light * L.area);
}

// ---------------------------------------------------------- environment ----
__device__ __forceinline__ f2 env_dir_to_uv(f3 wi) {  // light.rs:274-280
    float theta = acosf(clampf_(wi.y, -1.0f, 1.0f));
    float phi = atan2f(wi.z, wi.x);
    f2 uv; uv.x = (phi + PYRE_PI) * PYRE_FRAC_1_PI * 0.5f; uv.y = theta * PYRE_FRAC_1_PI;
    return uv;
}
__device__ __forceinline__ f3 env_uv_to_dir(f2 uv) {  // light.rs:282-287
    float phi = uv.x * PYRE_TAU - PYRE_PI;
    float theta = uv.y * PYRE_PI;
    float st, ct, sp, cp;
    sincosf(theta, &st, &ct);
    sincosf(phi, &sp, &cp);
    return mk3(st * cp, ct, st * sp);
}
__device__ __forceinline__ float fract_(float x) { return x - truncf(x); }
__device__ __forceinline__ int32_t sat_i32(float f) {  // Rust `as i32`
    if (isnan(f)) return 0;
    if (f >= 2147483647.0f) return 2147483647;
    if (f <= -2147483648.0f) return -2147483647 - 1;
    return (int32_t)f;
}
__device__ __forceinline__ uint32_t sat_usize(float f) {  // Rust `as usize` for the values seen here
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967295.0f) return 0xffffffffu;
    return (uint32_t)f;
}
__device__ __forceinline__ f3 env_texel(const DevEnv& E, uint32_t x, uint32_t y) {
    float4 p = __ldg(E.pixels + (size_t)y * E.width + x);
    return mk3(p.x, p.y, p.z);
}
__device__ __forceinline__ f3 env_texture(const DevEnv& E, f2 uv) {  // light.rs:290-314
    int32_t w = (int32_t)E.width, h = (int32_t)E.height;
    float u = fract_(fract_(uv.x) + 1.0f);
    float v = clampf_(uv.y, 0.0f, 1.0f);
    float fx = u * (float)w - 0.5f;
    float fy = clampf_(v * (float)h - 0.5f, 0.0f, (float)h - 1.0f);
    int32_t x0i = sat_i32(floorf(fx));
    int32_t y0i = sat_i32(floorf(fy));
    float dx = fx - (float)x0i;
    float dy = fy - (float)y0i;
    int32_t x0 = ((x0i % w) + w) % w;
    int32_t x1 = ((x0 + 1) % w + w) % w;
    int32_t y0 = min(max(y0i, 0), h - 1);
    int32_t y1 = min(y0 + 1, h - 1);
    f3 p00 = env_texel(E, x0, y0), p10 = env_texel(E, x1, y0), p01 = env_texel(E, x0, y1), p11 = env_texel(E, x1, y1);
    return p00 * ((1.0f - dx) * (1.0f - dy)) + p10 * (dx * (1.0f - dy)) + p01 * ((1.0f - dx) * dy) + p11 * (dx * dy);
}

// Distribution2D::pdf_at (distribution.rs:157-163) from per-bin pdf tables
// holding (cdf[b+1]-cdf[b])*n exactly as Distribution1D::pdf_at computes it.
__device__ __forceinline__ float env_pdf_uv(const DevEnv& E, f2 uv) {
    if (uv.x < 0.0f || uv.x >= 1.0f || uv.y < 0.0f || uv.y >= 1.0f) return 0.0f;
    uint32_t row = min(sat_usize(uv.y * (float)E.height), E.height - 1);
    uint32_t col = min(sat_usize(uv.x * (float)E.width), E.width - 1);
    return __ldg(E.cond_pdf + (size_t)row * E.width + col) * __ldg(E.marg_pdf + row);
}
// HdriEnvironmentLight::pdf (light.rs:340-349) at the texture coordinates of
// the direction.
__device__ __forceinline__ float env_pdf_at(const DevEnv& E, f2 uv) {
    float theta = uv.y * PYRE_PI;
    float st = sinf(theta);
    if (st < 1e-6f) return 0.0f;
    return env_pdf_uv(E, uv) / (2.0f * PYRE_PI * PYRE_PI * st);
}

// Distribution1D::sample_continuous (distribution.rs:79-101) over a CDF row.
__device__ __forceinline__ float cdf_sample(const float* cdf, uint32_t n, float u, float* pdf, uint32_t* bin_out) {
    uint32_t lo = 1, hi = n;
    while (lo < hi) {
        uint32_t mid = (lo + hi) / 2;
        if (__ldg(cdf + mid) <= u) lo = mid + 1; else hi = mid;
    }
    uint32_t bin = min(lo - 1, n - 1);
    float c0 = __ldg(cdf + bin), c1 = __ldg(cdf + bin + 1);
    float bin_size = fmaxf(c1 - c0, 1e-20f);
    float du = (u - c0) / bin_size;
    *pdf = bin_size * (float)n;
    *bin_out = bin;
    return ((float)bin + du) / (float)n;
}
// Alias-table draw of one continuous coordinate: the bin comes from the
// table (O(1), one dependent load), the offset inside the bin from the
// remaining fraction of u. The density is the reference's piecewise-constant
// pdf of the chosen bin.
__device__ __forceinline__ float alias_sample(const float2* table, const float* pdf_tab, uint32_t n, float u,
                                              float* pdf, uint32_t* bin_out) {
    float x = u * (float)n;
    uint32_t i = min((uint32_t)x, n - 1);
    float frac = x - (float)i;
    float2 e = __ldg(table + i);
    uint32_t bin;
    float du;
    if (frac < e.x) { bin = i; du = frac / e.x; }
    else { bin = __float_as_uint(e.y); du = (frac - e.x) / (1.0f - e.x); }
    du = fminf(du, 0.99999994f);
    *pdf = __ldg(pdf_tab + bin);
    *bin_out = bin;
    return ((float)bin + du) / (float)n;
}

// HdriEnvironmentLight::sample (light.rs:322-338).
__device__ __forceinline__ void env_sample(const DevEnv& E, f2 u, int cdf_mode, f3* wi, f3* li, float* pdf) {
    float pdf_v, pdf_u, v, uu;
    uint32_t row, col;
    if (cdf_mode) {
        v = cdf_sample(E.marg_cdf, E.height, u.y, &pdf_v, &row);
        uu = cdf_sample(E.cond_cdf + (size_t)row * (E.width + 1), E.width, u.x, &pdf_u, &col);
    } else {
        v = alias_sample(E.marg_alias, E.marg_pdf, E.height, u.y, &pdf_v, &row);
        uu = alias_sample(E.cond_alias + (size_t)row * E.width, E.cond_pdf + (size_t)row * E.width, E.width, u.x,
                          &pdf_u, &col);
    }
    f2 uv; uv.x = uu; uv.y = v;
    float pdf_uv = pdf_u * pdf_v;
    *wi = env_uv_to_dir(uv);
    float theta = uv.y * PYRE_PI;
    float st = sinf(theta);
    *pdf = (st > 1e-6f && pdf_uv > 0.0f) ? pdf_uv / (2.0f * PYRE_PI * PYRE_PI * st) : 0.0f;
    *li = env_texture(E, uv) * E.intensity;
}

// --------------------------------------------------------------- camera ----
struct DevCamera {
    f3 origin, forward, right, up;
    float half_width, half_height, aperture_radius, focus_distance;
    int thin_lens;
};
__device__ __forceinline__ f2 concentric_disk(f2 u) {  // distribution.rs:12-23
    f2 off; off.x = 2.0f * u.x - 1.0f; off.y = 2.0f * u.y - 1.0f;
    f2 z; z.x = 0.0f; z.y = 0.0f;
    if (off.x == 0.0f && off.y == 0.0f) return z;
    float r, theta;
    if (fabsf(off.x) > fabsf(off.y)) { r = off.x; theta = PYRE_FRAC_PI_4 * (off.y / off.x); }
    else { r = off.y; theta = PYRE_FRAC_PI_2 - PYRE_FRAC_PI_4 * (off.x / off.y); }
    float s, c;
    sincosf(theta, &s, &c);
    f2 o; o.x = r * c; o.y = r * s;
    return o;
}
// Camera::generate_ray (camera.rs:65-73 pinhole, 125-143 thin lens); Ray::new normalizes.
__device__ __forceinline__ void camera_ray(const DevCamera& C, f2 ndc, f2 lens, f3* o, f3* d) {
    f3 dir = C.forward + ndc.x * C.half_width * C.right + ndc.y * C.half_height * C.up;
    if (!C.thin_lens) {
        *o = C.origin;
        *d = normalize3(dir);
        return;
    }
    f3 pinhole_dir = normalize3(dir);
    float focal_t = C.focus_distance / dot3(pinhole_dir, C.forward);
    f3 focal_point = C.origin + focal_t * pinhole_dir;
    f2 disk = concentric_disk(lens);
    f3 lens_offset = C.aperture_radius * (disk.x * C.right + disk.y * C.up);
    f3 lens_origin = C.origin + lens_offset;
    *o = lens_origin;
    *d = normalize3(normalize3(focal_point - lens_origin));
}

// Host side.
inline DevCamera make_camera(const pyre_camera_desc& c) {
    // PinholeCamera / ThinLensCamera::look_at (camera.rs:49-72, 105-122) on the host.
    DevCamera d;
    f3 origin = mk3(c.origin[0], c.origin[1], c.origin[2]);
    f3 target = mk3(c.target[0], c.target[1], c.target[2]);
    f3 up = mk3(c.up[0], c.up[1], c.up[2]);
    d.origin = origin;
    d.forward = normalize3(target - origin);
    d.right = normalize3(cross3(d.forward, up));
    d.up = cross3(d.right, d.forward);
    const float to_rad = 3.14159265358979323846f / 180.0f;
    d.half_height = std::tan(c.vfov_deg * to_rad / 2.0f);
    d.half_width = c.aspect * d.half_height;
    d.aperture_radius = c.aperture_radius;
    d.focus_distance = c.focus_distance;
    d.thin_lens = c.kind == PYRE_CAMERA_THIN_LENS ? 1 : 0;
    return d;
}

}  // namespace pyre
