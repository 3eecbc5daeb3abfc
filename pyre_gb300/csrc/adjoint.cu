// adjoint.cu — path-replay adjoint of the path integrator.
//
// The reference has no differentiation; this is an addition. Gradients are
// taken of a scalar loss through the film, with respect to every material's
// (base color r,g,b, metallic, roughness, specular) and every environment
// texel, under the detached-sampling convention: only the BSDF values f (in
// the throughput and in NEE) and the emitted radiance carry derivatives;
// pdfs, MIS weights, lobe choice, Russian roulette and the environment's
// sampling tables are constants. Because the MIS weights of each direction
// sum to one, the estimator is unbiased for the derivative of the expected
// image.
//
// Path replay: every thread re-traces one path from its pixel seed
// (pixel_seed(x, y, s), the same Xoshiro draws and the same decisions as the
// forward wavefront), so no tape is stored between passes. During the replay
// the NEE and emission terms are differentiated on the spot (their
// throughput is known); the BSDF-sample term at vertex d needs the radiance
// arriving from the rest of the path, R_{d+1}, which a backward recursion
// R_d = t_d + g_d * R_{d+1} over a few floats per depth (kept in the thread's
// local memory) provides once the path has ended.
//
// Material gradients are summed per block in shared memory (FP64) and
// flushed with one FP64 atomic per parameter per block; texel gradients use
// FP32 atomics.
#include <algorithm>
#include <cstring>
#include <string>

#include "adjoint.cuh"
#include "internal.h"

namespace pyre {

#define PYRE_ADJ_MAXD 16
#define PYRE_ADJ_MAXSLOT 4

struct AdjParams {
    DevCamera cam;
    uint32_t width, height, cx0, cy0, cw, npix;
    uint32_t spp_begin, n_paths;
    uint32_t max_depth, min_rr;
    int env_cdf;
    float inv_spp;
    const float* dl_di;  // crop npix*3: d loss / d film radiance
    double* mat_grad;    // n_mat*6
    float* env_grad;     // env w*h*3 or null
    uint32_t n_mat;
    int smem_grad;       // material gradients summed in shared memory
};

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

// d(loss)/d(texel) for a radiance term c * Le(uv), Le = texture(uv) * intensity.
__device__ __forceinline__ void scatter_env(const DevEnv& E, float* env_grad, f2 uv, f3 c) {
    if (!env_grad) return;
    uint32_t idx[4];
    float wt[4];
    env_texel_weights(E, uv, idx, wt);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float s = wt[k] * E.intensity;
        if (s == 0.0f) continue;
        atomicAdd(env_grad + 3 * (size_t)idx[k], c.x * s);
        atomicAdd(env_grad + 3 * (size_t)idx[k] + 1, c.y * s);
        atomicAdd(env_grad + 3 * (size_t)idx[k] + 2, c.z * s);
    }
}

__device__ __forceinline__ void add_mat_grad(const AdjParams& A, double* sgrad, uint32_t m, const float g[6]) {
#pragma unroll
    for (int k = 0; k < PYRE_NPARAM; ++k) {
        if (g[k] == 0.0f) continue;
        if (A.smem_grad) atomicAdd(sgrad + PYRE_NPARAM * m + k, (double)g[k]);
        else atomicAdd(A.mat_grad + PYRE_NPARAM * (size_t)m + k, (double)g[k]);
    }
}

struct DepthRec {
    f3 wo, wi, beta, t, g;
    float a;
    int32_t mat;  // -1: no BSDF sample at this depth
};

__global__ void __launch_bounds__(128) k_adjoint(DevScene S, AdjParams A) {
    extern __shared__ double sgrad[];
    if (A.smem_grad)
        for (uint32_t k = threadIdx.x; k < A.n_mat * PYRE_NPARAM; k += blockDim.x) sgrad[k] = 0.0;
    __syncthreads();
    const unsigned FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t warp_global = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t ns = S.n_lights + (S.has_env ? 1u : 0u);
    const float INF = __int_as_float(0x7f800000);

    for (uint32_t base = warp_global * 32; base < A.n_paths; base += n_warps * 32) {
        const uint32_t i = base + lane;
        bool alive = i < A.n_paths;
        // ---- raygen (main.rs:261-273), as k_raygen
        Rng g;
        f3 ro = splat3(0.0f), rd = mk3(0.0f, 0.0f, 1.0f);
        float time = 0.0f;
        f3 delta = splat3(0.0f);
        if (alive) {
            const uint32_t k = i / A.npix, p = i - k * A.npix;
            const uint32_t x = A.cx0 + p % A.cw, y = A.cy0 + p / A.cw;
            g.seed(pixel_seed(x, y, A.spp_begin + k));
            float jx = g.next_f32(), jy = g.next_f32();
            f2 ndc;
            ndc.x = 2.0f * ((float)x + jx) / (float)A.width - 1.0f;
            ndc.y = 1.0f - 2.0f * ((float)y + jy) / (float)A.height;
            f2 lens = g.next_vec2();
            time = g.next_f32();
            camera_ray(A.cam, ndc, lens, &ro, &rd);
            delta = mk3(A.dl_di[3 * (size_t)p], A.dl_di[3 * (size_t)p + 1], A.dl_di[3 * (size_t)p + 2]) * A.inv_spp;
            if (is_zero3(delta)) alive = false;  // nothing to propagate for this pixel
        }
        f3 beta = splat3(1.0f);
        float last_pdf = 0.0f;
        DepthRec rec[PYRE_ADJ_MAXD];
        int nrec = 0;
        for (uint32_t depth = 0; depth < A.max_depth; ++depth) {
            if (!__any_sync(FULL, alive)) break;
            TraceRay r;
            r.o = ro; r.d = rd; r.tmin = 1e-4f; r.tmax = INF; r.time = time;
            TraceHit h;
            trace_closest_with_lights(S, r, alive, S.tlas_root, 0, S.n_lights, &h);
            // per-slot NEE set-up, traced below by the whole warp
            bool sh_valid[PYRE_ADJ_MAXSLOT];
            f3 sh_o[PYRE_ADJ_MAXSLOT], sh_d[PYRE_ADJ_MAXSLOT], nee_f[PYRE_ADJ_MAXSLOT], nee_c[PYRE_ADJ_MAXSLOT],
                nee_wi[PYRE_ADJ_MAXSLOT];
            float sh_tmax[PYRE_ADJ_MAXSLOT];
            f2 env_uv = {0.0f, 0.0f};
#pragma unroll
            for (int s = 0; s < PYRE_ADJ_MAXSLOT; ++s) sh_valid[s] = false;
            bool vertex = false, continue_path = false;
            Bsdf mat;
            mat.kind = 0;
            int32_t mat_id = -1;
            f3 wo = splat3(0.0f), t_d = splat3(0.0f), g_d = splat3(0.0f), wi_b = splat3(0.0f), beta_next = beta;
            float a_d = 0.0f;
            float env_k = 0.0f;  // env NEE factor wi.z * w / pdf (its texture term is differentiated)
            f3 next_o = ro, next_d = rd;
            if (alive) {
                if (h.inst < 0 && h.light < 0) {
                    // escaped: environment emission (integrator.rs:243-259)
                    if (S.has_env) {
                        f3 le = env_le(S.env, rd);
                        if (!is_zero3(le)) {
                            float w = 1.0f;
                            if (depth != 0) w = power_heuristic(last_pdf, env_pdf(S.env, rd));
                            t_d = le * w;
                            scatter_env(S.env, A.env_grad, env_dir_to_uv(rd), delta * beta * w);
                        }
                    }
                } else if (h.light >= 0) {
                    // quad light (integrator.rs:278-295)
                    const DevQuadLight& Lt = S.lights[h.light];
                    f3 le = dot3(Lt.normal, -rd) > 0.0f ? Lt.emission : splat3(0.0f);
                    float w = 1.0f;
                    if (depth != 0) w = power_heuristic(last_pdf, quad_pdf(Lt, ro, rd));
                    t_d = le * w;
                } else {
                    const DevInstance& I = S.inst[h.inst];
                    f3 off = splat3(0.0f);
                    if (I.has_motion) off = motion_offset(I, time);
                    const bool moved = !is_zero3(off);
                    f3 p = (moved ? ro - off : ro) + rd * h.t;
                    if (moved) p = p + off;
                    const float4 TA = __ldg(S.tris + 3 * (size_t)h.tri);
                    f3 nsh;
                    if (I.normal_base >= 0) {
                        const uint32_t* ix = S.index + I.index_base + 3 * (size_t)__float_as_uint(TA.w);
                        const f3 na = mk3(S.normal[3 * (size_t)ix[0]], S.normal[3 * (size_t)ix[0] + 1], S.normal[3 * (size_t)ix[0] + 2]);
                        const f3 nb = mk3(S.normal[3 * (size_t)ix[1]], S.normal[3 * (size_t)ix[1] + 1], S.normal[3 * (size_t)ix[1] + 2]);
                        const f3 nc = mk3(S.normal[3 * (size_t)ix[2]], S.normal[3 * (size_t)ix[2] + 1], S.normal[3 * (size_t)ix[2] + 2]);
                        const float w = 1.0f - h.u - h.v;
                        nsh = normalize3(w * na + h.u * nb + h.v * nc);
                    } else {
                        const float4 TB = __ldg(S.tris + 3 * (size_t)h.tri + 1), TC = __ldg(S.tris + 3 * (size_t)h.tri + 2);
                        nsh = normalize3(cross3(mk3(TB.x, TB.y, TB.z), mk3(TC.x, TC.y, TC.z)));
                    }
                    mat_id = (int32_t)I.material;
                    mat = load_bsdf(S, I.material);
                    const Frame3 fr = frame_from_normal(nsh);
                    wo = to_local(fr, -rd);
                    if (wo.z > 0.0f) {
                        vertex = true;
                        const f3 p_off = p + 1e-3f * nsh;
                        for (uint32_t l = 0; l < S.n_lights && l < PYRE_ADJ_MAXSLOT; ++l) {
                            f2 ul = g.next_vec2();
                            const DevQuadLight& Lt = S.lights[l];
                            f3 lpos, lwi;
                            float lpdf;
                            if (!quad_sample(Lt, p, ul, &lpos, &lwi, &lpdf)) continue;
                            if (lpdf <= 0.0f || is_zero3(Lt.emission)) continue;
                            f3 wi = to_local(fr, lwi);
                            if (wi.z <= 0.0f) continue;
                            f3 f = bsdf_eval(mat, wo, wi);
                            if (is_zero3(f)) continue;
                            f3 tf = (lpos - 1e-3f * lwi) - p_off;
                            float dist = len3(tf);
                            float w = power_heuristic(lpdf, bsdf_pdf(mat, wo, wi));
                            nee_f[l] = f;
                            nee_c[l] = Lt.emission * wi.z * w / lpdf;
                            nee_wi[l] = wi;
                            sh_valid[l] = true;
                            sh_o[l] = p_off;
                            if (dist > 0.0f) { sh_d[l] = tf / dist; sh_tmax[l] = dist - 1e-3f; }
                            else { sh_d[l] = mk3(0.0f, 0.0f, 1.0f); sh_tmax[l] = -1.0f; }  // visible, no ray
                        }
                        if (S.has_env) {
                            const uint32_t l = S.n_lights;
                            f2 ue = g.next_vec2();
                            f3 ewi, eli;
                            float epdf;
                            env_sample(S.env, ue, A.env_cdf, &ewi, &eli, &epdf);
                            if (epdf > 0.0f && !is_zero3(eli) && l < PYRE_ADJ_MAXSLOT) {
                                f3 wi = to_local(fr, ewi);
                                if (wi.z > 0.0f) {
                                    f3 f = bsdf_eval(mat, wo, wi);
                                    if (!is_zero3(f)) {
                                        float w = power_heuristic(epdf, bsdf_pdf(mat, wo, wi));
                                        env_k = wi.z * w / epdf;
                                        nee_f[l] = f;
                                        nee_c[l] = eli * env_k;
                                        nee_wi[l] = wi;
                                        sh_valid[l] = true;
                                        sh_o[l] = p_off; sh_d[l] = ewi; sh_tmax[l] = INF;
                                        env_uv = env_dir_to_uv(ewi);
                                    }
                                }
                            }
                        }
                        f3 bwi, bf;
                        float bpdf;
                        if (bsdf_sample(mat, wo, g.next_vec2(), &bwi, &bf, &bpdf) && bpdf > 0.0f && fabsf(bwi.z) != 0.0f) {
                            const float cos_wi = fabsf(bwi.z);
                            float a = cos_wi / bpdf;
                            f3 nb = beta * (bf * cos_wi / bpdf);
                            bool survive = true;
                            if (depth >= A.min_rr) {
                                float q = clampf_(1.0f - max_elem3(nb), 0.05f, 0.95f);
                                if (g.next_f32() < q) survive = false;
                                else { nb = nb / (1.0f - q); a = a / (1.0f - q); }
                            }
                            if (survive && depth + 1 < A.max_depth) {
                                continue_path = true;
                                wi_b = bwi;
                                a_d = a;
                                g_d = bf * a;
                                next_o = p_off;
                                next_d = to_world(fr, bwi);
                                last_pdf = bpdf;
                                beta_next = nb;  // applied after this vertex's terms
                            }
                        }
                    }
                }
            }
            // ---- visibility of the NEE rays, all lanes together (Scene::occluded)
            bool occl[PYRE_ADJ_MAXSLOT];
#pragma unroll
            for (int s = 0; s < PYRE_ADJ_MAXSLOT; ++s) {
                occl[s] = false;
                if (!__any_sync(FULL, sh_valid[s] && sh_tmax[s] >= 0.0f)) continue;
                TraceRay sr;
                const bool v = sh_valid[s] && sh_tmax[s] >= 0.0f;
                sr.o = v ? sh_o[s] : splat3(0.0f);
                sr.d = v ? sh_d[s] : mk3(0.0f, 0.0f, 1.0f);
                sr.tmin = 1e-3f; sr.tmax = v ? sh_tmax[s] : 0.0f; sr.time = time;
                TraceHit sh;
                occl[s] = trace_warp<true>(S, sr, v, S.tlas_root, &sh);
            }
            if (alive) {
                if (vertex) {
                    // NEE terms: value into t_d, derivatives right away (beta is beta_d)
                    for (uint32_t s = 0; s < ns && s < PYRE_ADJ_MAXSLOT; ++s) {
                        if (!sh_valid[s] || occl[s]) continue;
                        f3 c = nee_c[s];
                        t_d = t_d + nee_f[s] * c;
                        float J[3][PYRE_NPARAM];
                        bsdf_eval_jac(mat, wo, nee_wi[s], J);
                        const f3 wdb = delta * beta * c;
                        float gr[PYRE_NPARAM];
#pragma unroll
                        for (int k = 0; k < PYRE_NPARAM; ++k) gr[k] = wdb.x * J[0][k] + wdb.y * J[1][k] + wdb.z * J[2][k];
                        add_mat_grad(A, sgrad, (uint32_t)mat_id, gr);
                        if (S.has_env && s == S.n_lights) {
                            // term beta * f * (texture(uv) * intensity) * k: d/dtexel
                            scatter_env(S.env, A.env_grad, env_uv, delta * beta * nee_f[s] * env_k);
                        }
                    }
                }
                if (nrec < PYRE_ADJ_MAXD) {  // depth < max_depth <= PYRE_ADJ_MAXD
                    DepthRec& R = rec[nrec];
                    R.wo = wo; R.wi = wi_b; R.beta = beta; R.t = t_d;
                    R.g = continue_path ? g_d : splat3(0.0f);
                    R.a = a_d;
                    R.mat = (vertex && continue_path) ? mat_id : -1;
                    ++nrec;
                }
                if (continue_path) beta = beta_next;
                if (continue_path) { ro = next_o; rd = next_d; }
                else alive = false;
            }
        }
        // ---- backward recursion over depths: R_d = t_d + g_d * R_{d+1}
        f3 Rn = splat3(0.0f);
        for (int d = nrec - 1; d >= 0; --d) {
            const DepthRec& R = rec[d];
            if (R.mat >= 0 && !is_zero3(Rn)) {
                const DevMaterial M = S.materials[R.mat];
                Bsdf b;
                b.kind = M.kind; b.base = mk3(M.base[0], M.base[1], M.base[2]);
                b.metallic = M.metallic; b.roughness = M.roughness; b.specular = M.specular;
                float J[3][PYRE_NPARAM];
                bsdf_eval_jac(b, R.wo, R.wi, J);
                const f3 w = delta * R.beta * Rn * R.a;
                float gr[PYRE_NPARAM];
#pragma unroll
                for (int k = 0; k < PYRE_NPARAM; ++k) gr[k] = w.x * J[0][k] + w.y * J[1][k] + w.z * J[2][k];
                add_mat_grad(A, sgrad, (uint32_t)R.mat, gr);
            }
            Rn = R.t + R.g * Rn;
        }
    }
    __syncthreads();
    if (A.smem_grad)
        for (uint32_t k = threadIdx.x; k < A.n_mat * PYRE_NPARAM; k += blockDim.x)
            if (sgrad[k] != 0.0) atomicAdd(A.mat_grad + k, sgrad[k]);
}

}  // namespace pyre

using namespace pyre;

extern "C" int pyre_backward(pyre_ctx* ctx, const pyre_scene* scene, const pyre_camera_desc* camera,
                             const pyre_render_params* params, const float* d_loss_d_image, int image_mem,
                             pyre_gradients* grads) {
    if (!ctx || !scene || !camera || !params || !d_loss_d_image || !grads)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_backward: NULL argument");
    PYRE_CUDA_TRY(ctx, cudaSetDevice(ctx->device));
    const pyre_render_params& rp = *params;
    if (rp.width == 0 || rp.height == 0) return set_error(ctx, PYRE_ERR_INVALID, "image size is zero");
    if (rp.spp_end <= rp.spp_begin) return set_error(ctx, PYRE_ERR_INVALID, "empty sample range");
    if (rp.max_depth > PYRE_ADJ_MAXD) return set_error(ctx, PYRE_ERR_INVALID, "pyre_backward: max_depth above 16");
    if (scene->n_parts != 1) return set_error(ctx, PYRE_ERR_UNSUPPORTED, "pyre_backward: batched scenes");
    const uint32_t ns = scene->dev.n_lights + (scene->dev.has_env ? 1u : 0u);
    if (ns > PYRE_ADJ_MAXSLOT) return set_error(ctx, PYRE_ERR_UNSUPPORTED, "pyre_backward: more than 3 quad lights");
    if (image_mem != PYRE_MEM_HOST && image_mem != PYRE_MEM_DEVICE) return set_error(ctx, PYRE_ERR_INVALID, "bad image_mem");
    if (grads->mem != PYRE_MEM_HOST && grads->mem != PYRE_MEM_DEVICE) return set_error(ctx, PYRE_ERR_INVALID, "bad grads.mem");
    uint32_t x0 = rp.crop[0], y0 = rp.crop[1], x1 = rp.crop[2], y1 = rp.crop[3];
    if (x0 == 0 && y0 == 0 && x1 == 0 && y1 == 0) { x1 = rp.width; y1 = rp.height; }
    if (x1 > rp.width || y1 > rp.height || x0 >= x1 || y0 >= y1)
        return set_error(ctx, PYRE_ERR_INVALID, "crop outside the image");

    AdjParams A;
    std::memset(&A, 0, sizeof A);
    A.cam = make_camera(*camera);
    A.width = rp.width; A.height = rp.height;
    A.cx0 = x0; A.cy0 = y0; A.cw = x1 - x0;
    A.npix = A.cw * (y1 - y0);
    A.spp_begin = rp.spp_begin;
    const uint64_t n_paths = (uint64_t)A.npix * (rp.spp_end - rp.spp_begin);
    if (n_paths > 0xffffffffull) return set_error(ctx, PYRE_ERR_INVALID, "pyre_backward: too many paths");
    A.n_paths = (uint32_t)n_paths;
    A.max_depth = rp.max_depth; A.min_rr = rp.min_rr_depth;
    A.env_cdf = rp.env_sampling == PYRE_ENV_CDF ? 1 : 0;
    A.inv_spp = 1.0f / (float)(rp.spp_end - rp.spp_begin);
    A.n_mat = scene->dev.n_materials;
    const size_t mat_bytes = (size_t)A.n_mat * PYRE_NPARAM * sizeof(double);
    const size_t env_elems = scene->dev.has_env ? (size_t)scene->dev.env.width * scene->dev.env.height * 3 : 0;
    const size_t img_bytes = (size_t)A.npix * 3 * sizeof(float);
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    int rc = ensure_workspace(ctx, ctx->io_ws, al(mat_bytes) + al(env_elems * 4) + al(img_bytes) + 256);
    if (rc) return rc;
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
    A.dl_di = d_img;
    A.mat_grad = d_mat;
    A.env_grad = (env_elems && grads->env) ? d_env : nullptr;
    const size_t smem = mat_bytes <= 48 * 1024 ? mat_bytes : 0;
    A.smem_grad = smem ? 1 : 0;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adjoint, 128, smem);
    const int grid = std::max(1, per_sm) * std::max(1, ctx->num_sms);
    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[0], st));
    k_adjoint<<<grid, 128, smem, st>>>(scene->dev, A);
    PYRE_CUDA_TRY(ctx, cudaGetLastError());
    PYRE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev[1], st));
    if (grads->mem == PYRE_MEM_HOST) {
        if (grads->materials && mat_bytes)
            PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(grads->materials, d_mat, mat_bytes, cudaMemcpyDeviceToHost, st));
        if (grads->env && env_elems)
            PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(grads->env, d_env, env_elems * 4, cudaMemcpyDeviceToHost, st));
    }
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    if ((rc = take_kernel_error(ctx))) return rc;
    std::memset(&ctx->stats, 0, sizeof ctx->stats);
    ctx->stats.samples = n_paths;
    ctx->stats.kernel_launches = 1;
    cudaEventElapsedTime(&ctx->stats.ms_total, ctx->ev[0], ctx->ev[1]);
    return PYRE_OK;
}
