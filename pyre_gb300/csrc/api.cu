// api.cu — context, errors and scene upload of the C ABI.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <thread>

#include "bvh_host.h"
#include "internal.h"
#include "shading.cuh"

namespace pyre {

static thread_local std::string g_tls_error;

int set_error(pyre_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->error = msg;
    else g_tls_error = msg;
    return code;
}

int cuda_check(pyre_ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return PYRE_OK;
    std::string msg = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return set_error(ctx, e == cudaErrorMemoryAllocation ? PYRE_ERR_OOM : PYRE_ERR_CUDA, msg);
}

bool injected_alloc_failure(pyre_ctx* ctx) {
    if (!ctx || ctx->fail_alloc_countdown < 0) return false;
    if (ctx->fail_alloc_countdown == 0) {
        ctx->fail_alloc_countdown = -1;
        return true;
    }
    --ctx->fail_alloc_countdown;
    return false;
}

int ensure_workspace(pyre_ctx* ctx, Workspace& ws, size_t bytes) {
    if (ws.bytes >= bytes) return PYRE_OK;
    if (ws.ptr) {
        cudaFree(ws.ptr);
        ws.ptr = nullptr;
        ws.bytes = 0;
    }
    // Any cached wave graph refers to the old buffers.
    if (ctx->wave_graph) {
        cudaGraphExecDestroy(ctx->wave_graph);
        ctx->wave_graph = nullptr;
        ctx->wave_graph_key.clear();
    }
    if (injected_alloc_failure(ctx))
        return set_error(ctx, PYRE_ERR_OOM, "cudaMalloc(workspace): injected allocation failure");
    size_t rounded = (bytes + (1u << 20) - 1) & ~(size_t)((1u << 20) - 1);
    cudaError_t e = cudaMalloc(&ws.ptr, rounded);
    if (e != cudaSuccess) {
        ws.ptr = nullptr;
        cudaGetLastError();  // an allocation failure is not sticky: clear it for the next launch checks
        return cuda_check(ctx, e, "cudaMalloc(workspace)");
    }
    ws.bytes = rounded;
    return PYRE_OK;
}

int take_kernel_error(pyre_ctx* ctx) {
    int flag = 0;
    cudaError_t e = cudaMemcpyAsync(&flag, ctx->d_error, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_check(ctx, e, "reading the kernel status");
    if (flag != 0) {
        cudaMemsetAsync(ctx->d_error, 0, sizeof(int), ctx->stream);
        cudaStreamSynchronize(ctx->stream);
        if (flag == PYRE_ERR_OVERFLOW)
            return set_error(ctx, PYRE_ERR_OVERFLOW, "a kernel hit its traversal-stack or queue limit");
        return set_error(ctx, flag, "a kernel reported an error status");
    }
    return PYRE_OK;
}

namespace {

template <typename T>
int upload(pyre_ctx* ctx, pyre_scene* sc, const std::vector<T>& host, T** out) {
    *out = nullptr;
    if (host.empty()) return PYRE_OK;
    void* p = nullptr;
    size_t bytes = host.size() * sizeof(T);
    if (injected_alloc_failure(ctx))
        return set_error(ctx, PYRE_ERR_OOM, "cudaMalloc(scene): injected allocation failure");
    cudaError_t e = cudaMalloc(&p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return cuda_check(ctx, e, "cudaMalloc(scene)");
    }
    sc->allocations.push_back(p);
    sc->device_bytes += bytes;
    e = cudaMemcpy(p, host.data(), bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_check(ctx, e, "cudaMemcpy(scene)");
    *out = (T*)p;
    return PYRE_OK;
}

// Distribution1D (distribution.rs:40-61) in binary32: running sum of max(w,0),
// normalised by the integral, uniform when the integral is not positive.
float build_cdf(const float* w, uint32_t n, float* cdf) {
    cdf[0] = 0.0f;
    float acc = 0.0f;
    for (uint32_t i = 0; i < n; ++i) {
        acc += std::fmax(w[i], 0.0f);
        cdf[i + 1] = acc;
    }
    if (acc > 0.0f) {
        for (uint32_t i = 0; i <= n; ++i) cdf[i] /= acc;
    } else {
        for (uint32_t i = 0; i <= n; ++i) cdf[i] = (float)i / (float)n;
    }
    return acc;
}

// Vose's alias method over bin probabilities taken from the CDF differences.
void build_alias(const float* cdf, uint32_t n, float2* table) {
    std::vector<double> q(n);
    double sum = 0.0;
    for (uint32_t i = 0; i < n; ++i) {
        q[i] = std::max(0.0, (double)cdf[i + 1] - (double)cdf[i]);
        sum += q[i];
    }
    std::vector<uint32_t> small, large;
    std::vector<double> scaled(n);
    for (uint32_t i = 0; i < n; ++i) {
        scaled[i] = sum > 0.0 ? q[i] * (double)n / sum : 1.0;
        (scaled[i] < 1.0 ? small : large).push_back(i);
        table[i].x = 1.0f;
        uint32_t self = i;
        std::memcpy(&table[i].y, &self, 4);
    }
    while (!small.empty() && !large.empty()) {
        uint32_t s = small.back(); small.pop_back();
        uint32_t l = large.back(); large.pop_back();
        table[s].x = (float)scaled[s];
        std::memcpy(&table[s].y, &l, 4);
        scaled[l] = (scaled[l] + scaled[s]) - 1.0;
        (scaled[l] < 1.0 ? small : large).push_back(l);
    }
    for (uint32_t i : small) table[i].x = 1.0f;
    for (uint32_t i : large) table[i].x = 1.0f;
}

// Environment texels and sampling tables of HdriEnvironmentLight::new
// (light.rs:214-242): weights lum * sin(theta_row), Distribution2D CDFs,
// per-bin pdfs and alias tables.
struct EnvTables {
    std::vector<float4> px;
    std::vector<float> marg_cdf, cond_cdf, marg_pdf, cond_pdf;
    std::vector<float2> marg_alias, cond_alias;
};

// Distribution2D (distribution.rs:113-172) over w x h weights: conditional
// CDFs per row, marginal CDF over the row integrals, per-bin pdfs, alias tables.
void build_dist2d(uint32_t w, uint32_t h, const float* weights, EnvTables& t) {
    t.cond_cdf.resize((size_t)h * (w + 1));
    t.cond_pdf.resize((size_t)w * h);
    t.cond_alias.resize((size_t)w * h);
    std::vector<float> row_integral(h);
    for (uint32_t y = 0; y < h; ++y) {
        float* cdf = t.cond_cdf.data() + (size_t)y * (w + 1);
        row_integral[y] = build_cdf(weights + (size_t)y * w, w, cdf);
        for (uint32_t x = 0; x < w; ++x) t.cond_pdf[(size_t)y * w + x] = (cdf[x + 1] - cdf[x]) * (float)w;
        build_alias(cdf, w, t.cond_alias.data() + (size_t)y * w);
    }
    t.marg_cdf.resize(h + 1);
    t.marg_pdf.resize(h);
    t.marg_alias.resize(h);
    build_cdf(row_integral.data(), h, t.marg_cdf.data());
    for (uint32_t y = 0; y < h; ++y) t.marg_pdf[y] = (t.marg_cdf[y + 1] - t.marg_cdf[y]) * (float)h;
    build_alias(t.marg_cdf.data(), h, t.marg_alias.data());
}

void build_env_tables(uint32_t w, uint32_t h, const float* rgb, EnvTables& t) {
    t.px.resize((size_t)w * h);
    std::vector<float> weights((size_t)w * h);
    for (uint32_t y = 0; y < h; ++y) {
        float theta = ((float)y + 0.5f) / (float)h * 3.14159265358979323846f;
        float sin_theta = std::fmax(std::sin(theta), 0.0f);
        for (uint32_t x = 0; x < w; ++x) {
            const float* p = rgb + 3 * ((size_t)y * w + x);
            t.px[(size_t)y * w + x] = make_float4(p[0], p[1], p[2], 0.0f);
            float lum = 0.21267f * p[0] + 0.71516f * p[1] + 0.07217f * p[2];
            weights[(size_t)y * w + x] = std::fmax(lum, 0.0f) * sin_theta;
        }
    }
    build_dist2d(w, h, weights.data(), t);
}

// ------------------------------------------------------ device queries --
// Distribution2D::sample / pdf (distribution.rs:139-172) through the device
// code the environment light uses: out_s gets (u, v, pdf, column, row) per
// draw, out_p the piecewise-constant pdf at each uv.
__global__ void k_dist2d_query(DevEnv E, int cdf_mode, const float* __restrict__ u, uint32_t n,
                               const float* __restrict__ uv, uint32_t m, float* out_s, float* out_p) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        float pu, pv, x, y;
        uint32_t row, col;
        if (cdf_mode) {
            y = cdf_sample(E.marg_cdf, E.height, u[2 * i + 1], &pv, &row);
            x = cdf_sample(E.cond_cdf + (size_t)row * (E.width + 1), E.width, u[2 * i], &pu, &col);
        } else {
            y = alias_sample(E.marg_alias, E.marg_pdf, E.height, u[2 * i + 1], &pv, &row);
            x = alias_sample(E.cond_alias + (size_t)row * E.width, E.cond_pdf + (size_t)row * E.width, E.width,
                             u[2 * i], &pu, &col);
        }
        float* o = out_s + 5 * (size_t)i;
        o[0] = x; o[1] = y; o[2] = pu * pv; o[3] = (float)col; o[4] = (float)row;
    }
    if (i < m) {
        f2 q; q.x = uv[2 * i]; q.y = uv[2 * i + 1];
        out_p[i] = env_pdf_uv(E, q);
    }
}

// Per triangle slot, the global vertex ids of its triangle (rows of the
// rebased index buffer, which also index the normal array):
// index[index_base(mesh) + 3 * local id], the local id being the triangle
// record's .w. Slots run mesh by mesh; mesh k holds slots
// [slot_start[k], slot_start[k + 1]).
// The three vertex normals of each triangle slot, in BVH leaf order (zero for
// meshes without normals, whose shading normal comes from the edges): shade
// reads a hit's normals with three loads from one 48-B record that does not
// wait for the instance, instead of a vertex-id record and nine loads that
// wait on it (shade 43.5 against 44.7 ms on the 1080p studio frame).
__global__ void k_slot_normals(const float4* __restrict__ tris, const uint32_t* __restrict__ index,
                               const float* __restrict__ normal, const uint32_t* __restrict__ slot_start,
                               const uint32_t* __restrict__ index_base, const uint8_t* __restrict__ has_normals,
                               uint32_t n_mesh, uint32_t n_slots, float4* __restrict__ out) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n_slots; t += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n_mesh - 1;  // last mesh with slot_start <= t
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) / 2;
            if (slot_start[mid] <= t) lo = mid; else hi = mid - 1;
        }
        const size_t row = index_base[lo] + 3 * (size_t)__float_as_uint(tris[3 * (size_t)t].w);
        for (int k = 0; k < 3; ++k) {
            float4 n = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            if (has_normals[lo]) {
                const size_t a = 3 * (size_t)index[row + k];
                n = make_float4(normal[a], normal[a + 1], normal[a + 2], 0.0f);
            }
            out[3 * (size_t)t + k] = n;
        }
    }
}

// BsdfSample / eval / pdf (material.rs:42-226) per (wo, u): out gets
// (sampled, wi.xyz, f.xyz, pdf, eval(wo, wi).xyz, pdf(wo, wi)).
__global__ void k_bsdf_query(Bsdf b, const float* __restrict__ wo, const float* __restrict__ u, uint32_t n,
                             float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f3 w = mk3(wo[3 * (size_t)i], wo[3 * (size_t)i + 1], wo[3 * (size_t)i + 2]);
    f2 q; q.x = u[2 * (size_t)i]; q.y = u[2 * (size_t)i + 1];
    f3 wi = splat3(0.0f), f = splat3(0.0f), fe = splat3(0.0f);
    float pdf = 0.0f, pe = 0.0f;
    const bool ok = bsdf_sample(b, w, q, &wi, &f, &pdf);
    if (ok) { fe = bsdf_eval(b, w, wi); pe = bsdf_pdf(b, w, wi); }
    float* o = out + 13 * (size_t)i;
    o[0] = ok ? 1.0f : 0.0f;
    o[1] = wi.x; o[2] = wi.y; o[3] = wi.z;
    o[4] = f.x; o[5] = f.y; o[6] = f.z; o[7] = pdf;
    o[8] = fe.x; o[9] = fe.y; o[10] = fe.z; o[11] = pe;
    o[12] = 0.0f;
}

std::atomic<uint64_t> g_scene_serial{1};

}  // namespace
}  // namespace pyre

using namespace pyre;

extern "C" {

int pyre_version(void) { return PYRE_ABI_VERSION; }

const char* pyre_last_error(const pyre_ctx* ctx) {
    return ctx ? ctx->error.c_str() : g_tls_error.c_str();
}

int pyre_ctx_create(int device, pyre_ctx** out) {
    if (!out) return set_error(nullptr, PYRE_ERR_INVALID, "pyre_ctx_create: out is NULL");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_check(nullptr, e, "cudaGetDeviceCount");
    if (device < 0 || device >= count) return set_error(nullptr, PYRE_ERR_INVALID, "pyre_ctx_create: no such device");
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_check(nullptr, e, "cudaSetDevice");
    pyre_ctx* ctx = new pyre_ctx();
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaMalloc(&ctx->d_error, sizeof(int))) != cudaSuccess ||
        (e = cudaMalloc(&ctx->d_counter, 64 * sizeof(unsigned int))) != cudaSuccess ||
        (e = cudaMemset(ctx->d_error, 0, sizeof(int))) != cudaSuccess) {
        int rc = cuda_check(nullptr, e, "pyre_ctx_create");
        pyre_ctx_destroy(ctx);
        return rc;
    }
    for (auto& ev : ctx->ev) cudaEventCreate(&ev);
    *out = ctx;
    return PYRE_OK;
}

int pyre_ctx_destroy(pyre_ctx* ctx) {
    if (!ctx) return PYRE_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->wave_graph) cudaGraphExecDestroy(ctx->wave_graph);
    if (ctx->render_ws.ptr) cudaFree(ctx->render_ws.ptr);
    if (ctx->io_ws.ptr) cudaFree(ctx->io_ws.ptr);
    if (ctx->tape_ws.ptr) cudaFree(ctx->tape_ws.ptr);
    if (ctx->prog_ws.ptr) cudaFree(ctx->prog_ws.ptr);
    if (ctx->d_error) cudaFree(ctx->d_error);
    if (ctx->d_counter) cudaFree(ctx->d_counter);
    for (auto& ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : ctx->stage_ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : ctx->wave_ev) cudaEventDestroy(ev);
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return PYRE_OK;
}

int pyre_scene_destroy(pyre_ctx* ctx, pyre_scene* scene) {
    if (!scene) return PYRE_OK;
    if (ctx) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    for (void* p : scene->allocations) cudaFree(p);
    delete scene;
    return PYRE_OK;
}

}  // extern "C"

// Uploads `desc` as n_parts independent sub-scenes sharing one device scene:
// instance i and light l belong to part inst_part[i] / light_part[l] (lights
// grouped by part, in part order). Each part gets its own top-level BVH and
// light range, so rays of one part never see another part's geometry.
static int upload_parts(pyre_ctx* ctx, const pyre_scene_desc* desc, const std::vector<uint32_t>& inst_part,
                        const std::vector<uint32_t>& light_part, uint32_t n_parts, pyre_scene** out) {
    if (!ctx || !desc || !out) return set_error(ctx, PYRE_ERR_INVALID, "pyre_scene_upload: NULL argument");
    *out = nullptr;
    cudaSetDevice(ctx->device);
    const uint32_t n_meshes = desc->n_meshes;
    if (n_meshes && !desc->meshes) return set_error(ctx, PYRE_ERR_INVALID, "meshes is NULL");
    if (desc->n_instances && !desc->instances) return set_error(ctx, PYRE_ERR_INVALID, "instances is NULL");
    if (desc->n_materials && !desc->materials) return set_error(ctx, PYRE_ERR_INVALID, "materials is NULL");
    if (desc->n_lights && !desc->lights) return set_error(ctx, PYRE_ERR_INVALID, "lights is NULL");

    // ---- validate meshes and instances
    for (uint32_t m = 0; m < n_meshes; ++m) {
        const pyre_mesh_desc& md = desc->meshes[m];
        if (md.n_triangles && (!md.positions || !md.indices))
            return set_error(ctx, PYRE_ERR_INVALID, "mesh " + std::to_string(m) + ": positions/indices NULL");
        for (uint64_t i = 0; i < 3ull * md.n_triangles; ++i)
            if (md.indices[i] >= md.n_vertices)
                return set_error(ctx, PYRE_ERR_INVALID, "mesh " + std::to_string(m) + ": vertex index out of range");
        if (md.bvh_nodes) {
            std::string why;
            if (!validate_bvh2(md.bvh_nodes, md.n_bvh_nodes, md.bvh_prim_indices, md.n_triangles, &why))
                return set_error(ctx, PYRE_ERR_INVALID, "mesh " + std::to_string(m) + ": " + why);
        }
    }
    for (uint32_t i = 0; i < desc->n_instances; ++i) {
        const pyre_instance_desc& id = desc->instances[i];
        if (id.mesh >= n_meshes) return set_error(ctx, PYRE_ERR_INVALID, "instance mesh out of range");
        if (id.material >= desc->n_materials)
            return set_error(ctx, PYRE_ERR_INVALID, "instance material out of range");
    }
    for (uint32_t i = 0; i < desc->n_materials; ++i)
        if (desc->materials[i].kind > PYRE_MAT_DISNEY) return set_error(ctx, PYRE_ERR_INVALID, "unknown material kind");
    if (desc->env && (desc->env->width == 0 || desc->env->height == 0 || !desc->env->rgb))
        return set_error(ctx, PYRE_ERR_INVALID, "environment map is empty");

    // ---- per-mesh reference BVH2 (caller's, or built here in parallel on the
    // host threads, or built for all meshes at once on the GPU)
    bool device_build = ctx->bvh_builder == PYRE_BVH_BUILDER_DEVICE;
    for (uint32_t m = 0; m < n_meshes; ++m)
        if (desc->meshes[m].bvh_nodes) device_build = false;
    std::vector<std::vector<pyre_bvh2_node>> built(n_meshes);
    std::vector<std::vector<uint32_t>> built_prim(n_meshes);
    if (!device_build) {
        std::atomic<uint32_t> next{0};
        auto work = [&]() {
            for (uint32_t m = next++; m < n_meshes; m = next++) {
                const pyre_mesh_desc& md = desc->meshes[m];
                if (md.bvh_nodes || md.n_triangles == 0) continue;
                std::vector<Aabb> b;
                std::vector<f3> c;
                triangle_bounds(md.positions, md.indices, md.n_triangles, b, c);
                build_bvh2(b, c, built[m], built_prim[m]);
            }
        };
        unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 32u));
        nt = std::min<unsigned>(nt, std::max<uint32_t>(n_meshes, 1));
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < nt; ++t) pool.emplace_back(work);
        work();
        for (auto& t : pool) t.join();
    }

    pyre_scene* sc = new pyre_scene();
    sc->serial = g_scene_serial++;
    auto fail = [&](int rc) { pyre_scene_destroy(ctx, sc); return rc; };

    // ---- collapse BVHs, lay out triangle slots, index and normal buffers
    std::vector<GpuNode> nodes;
    std::vector<float4> tris;
    std::vector<uint32_t> index;
    std::vector<float> normal;
    std::vector<int32_t> mesh_root(n_meshes, -1), mesh_index_base(n_meshes, 0), mesh_normal_base(n_meshes, -1);
    std::vector<Aabb> mesh_box(n_meshes);
    uint64_t total_tris = 0, total_verts_n = 0;
    for (uint32_t m = 0; m < n_meshes; ++m) {
        total_tris += desc->meshes[m].n_triangles;
        if (desc->meshes[m].normals) total_verts_n += desc->meshes[m].n_vertices;
    }
    if (total_tris > (uint64_t)INT32_MAX / 3) return fail(set_error(ctx, PYRE_ERR_INVALID, "too many triangles"));
    tris.reserve(3 * total_tris);
    index.reserve(3 * total_tris);
    normal.reserve(3 * total_verts_n);
    std::vector<uint32_t> device_meshes;  // meshes with triangles, in slot order
    for (uint32_t m = 0; m < n_meshes; ++m) {
        const pyre_mesh_desc& md = desc->meshes[m];
        mesh_index_base[m] = (int32_t)index.size();
        if (md.n_triangles == 0) continue;
        if (device_build) {
            device_meshes.push_back(m);
        } else {
            const pyre_bvh2_node* bn = md.bvh_nodes ? md.bvh_nodes : built[m].data();
            uint32_t nn = md.bvh_nodes ? md.n_bvh_nodes : (uint32_t)built[m].size();
            const uint32_t* prim = md.bvh_nodes ? md.bvh_prim_indices : built_prim[m].data();
            int32_t slot_base = (int32_t)(tris.size() / 3);
            mesh_root[m] = (int32_t)nodes.size();
            mesh_box[m] = collapse_bvh2(bn, nn, (int32_t)nodes.size(), slot_base, nodes);
            for (uint32_t k = 0; k < md.n_triangles; ++k) {
                uint32_t t = prim[k];
                const float* p0 = md.positions + 3 * (size_t)md.indices[3 * (size_t)t];
                const float* p1 = md.positions + 3 * (size_t)md.indices[3 * (size_t)t + 1];
                const float* p2 = md.positions + 3 * (size_t)md.indices[3 * (size_t)t + 2];
                float id_bits;
                std::memcpy(&id_bits, &t, 4);
                tris.push_back(make_float4(p0[0], p0[1], p0[2], id_bits));
                tris.push_back(make_float4(p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2], 0.0f));
                tris.push_back(make_float4(p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2], 0.0f));
            }
        }
        uint32_t vbase = md.normals ? (uint32_t)(normal.size() / 3) : 0;
        if (md.normals) {
            mesh_normal_base[m] = (int32_t)vbase;
            normal.insert(normal.end(), md.normals, md.normals + 3 * (size_t)md.n_vertices);
        }
        for (uint64_t i = 0; i < 3ull * md.n_triangles; ++i) index.push_back(vbase + md.indices[i]);
    }

    // instance BVHs built on the GPU: nodes and triangle records stay on the device
    DeviceBlas blas;
    struct FreeNodes {  // the device-built nodes until they are copied into the scene
        DeviceBlas& b;
        ~FreeNodes() { if (b.nodes) cudaFree(b.nodes); }
    } free_nodes{blas};
    if (device_build && !device_meshes.empty()) {
        const int rc0 = device_build_blas(ctx, desc, device_meshes, &blas);
        if (rc0) return fail(rc0);
        sc->allocations.push_back(blas.tris);
        sc->device_bytes += 3 * total_tris * sizeof(float4);
        for (size_t k = 0; k < device_meshes.size(); ++k) {
            mesh_root[device_meshes[k]] = blas.root[k];
            mesh_box[device_meshes[k]] = blas.box[k];
        }
    }
    const int32_t node_off = (int32_t)blas.n_nodes;  // top-level nodes follow the device-built ones

    // ---- instances and one top-level BVH per part over their swept bounds
    std::vector<DevInstance> inst;
    std::vector<int32_t> part_tlas(n_parts, -1);
    sc->slot_of_instance.assign(desc->n_instances, -1);
    for (uint32_t part = 0; part < n_parts; ++part) {
        std::vector<uint32_t> live;  // instances of this part with geometry
        std::vector<Aabb> ibox;
        std::vector<f3> icent;
        for (uint32_t i = 0; i < desc->n_instances; ++i) {
            if (inst_part[i] != part) continue;
            const pyre_instance_desc& id = desc->instances[i];
            if (mesh_root[id.mesh] < 0) continue;
            Aabb base = mesh_box[id.mesh];
            Aabb w = base;
            if (id.has_motion) {  // MeshInstance::world_bounds, mesh.rs:95-105
                f3 o0 = mk3(id.offset_t0[0], id.offset_t0[1], id.offset_t0[2]);
                f3 o1 = mk3(id.offset_t1[0], id.offset_t1[1], id.offset_t1[2]);
                w.lo = vmin3(base.lo + o0, base.lo + o1);
                w.hi = vmax3(base.hi + o0, base.hi + o1);
            }
            // The top level is an addition of this library: pad it so its test is
            // never tighter than the reference's per-instance root test.
            float mag = std::max({std::fabs(w.lo.x), std::fabs(w.lo.y), std::fabs(w.lo.z), std::fabs(w.hi.x),
                                  std::fabs(w.hi.y), std::fabs(w.hi.z), 1e-3f});
            if (id.has_motion)
                for (int k = 0; k < 3; ++k)
                    mag = std::max({mag, std::fabs(id.offset_t0[k]), std::fabs(id.offset_t1[k])});
            float pad = mag * 1e-5f;
            w.lo = w.lo - splat3(pad);
            w.hi = w.hi + splat3(pad);
            live.push_back(i);
            ibox.push_back(w);
            icent.push_back((w.lo + w.hi) * 0.5f);
        }
        if (live.empty()) continue;
        std::vector<pyre_bvh2_node> tn;
        std::vector<uint32_t> tp;
        build_bvh2(ibox, icent, tn, tp, PYRE_TLAS_ENTER ? 1u : 8u);
        const int32_t slot_base = (int32_t)inst.size();
        part_tlas[part] = node_off + (int32_t)nodes.size();
        const size_t first_top = nodes.size();
        collapse_bvh2(tn.data(), (uint32_t)tn.size(), node_off + (int32_t)nodes.size(), slot_base, nodes);
        // A top-level leaf of one static instance holds that instance's root
        // box, unpadded, and the child entry INST|TOP|slot with count -1: the
        // top-level step's test of the box is the reference's root test
        // (bvh.rs:103-110) and the lane then enters the instance without a
        // node step of its own.
        for (size_t g = first_top; PYRE_TLAS_ENTER && g < nodes.size(); ++g)
            for (int c = 0; c < 2; ++c) {
                if (nodes[g].d[2 + c] != 1) continue;
                const int32_t slot = nodes[g].d[c];
                const pyre_instance_desc& id = desc->instances[live[tp[(size_t)(slot - slot_base)]]];
                if (id.has_motion) continue;
                set_gpu_child(nodes[g], c, mesh_box[id.mesh], slot | PYRE_TAG_INST | PYRE_TAG_TOP, -1);
            }
        inst.resize(inst.size() + tp.size());
        for (size_t k = 0; k < tp.size(); ++k) {
            uint32_t i = live[tp[k]];
            const pyre_instance_desc& id = desc->instances[i];
            DevInstance& I = inst[slot_base + k];
            std::memset(&I, 0, sizeof I);
            const Aabb& rb = mesh_box[id.mesh];
            I.lo[0] = rb.lo.x; I.lo[1] = rb.lo.y; I.lo[2] = rb.lo.z;
            I.hi[0] = rb.hi.x; I.hi[1] = rb.hi.y; I.hi[2] = rb.hi.z;
            I.blas_root = mesh_root[id.mesh];
            I.has_motion = id.has_motion ? 1 : 0;
            for (int c = 0; c < 3; ++c) { I.off0[c] = id.offset_t0[c]; I.off1[c] = id.offset_t1[c]; }
            I.orig_id = (int32_t)i;
            I.mesh = (int32_t)id.mesh;
            I.material = id.material;
            I.index_base = (uint32_t)mesh_index_base[id.mesh];
            I.normal_base = mesh_normal_base[id.mesh];
            I.tri_count = desc->meshes[id.mesh].n_triangles;
            sc->slot_of_instance[i] = slot_base + (int32_t)k;
        }
    }
    const int32_t tlas_root = part_tlas[0];
    // per-part light ranges (first, count)
    std::vector<uint32_t> part_light(2 * n_parts, 0);
    for (uint32_t l = 0; l < desc->n_lights; ++l) {
        uint32_t pp = light_part[l];
        if (part_light[2 * pp + 1] == 0) part_light[2 * pp] = l;
        part_light[2 * pp + 1] += 1;
    }

    // ---- materials and lights
    std::vector<DevMaterial> mats(desc->n_materials);
    for (uint32_t i = 0; i < desc->n_materials; ++i) {
        const pyre_material_desc& m = desc->materials[i];
        DevMaterial& d = mats[i];
        for (int c = 0; c < 3; ++c) d.base[c] = m.base_color[c];
        d.kind = m.kind; d.metallic = m.metallic; d.roughness = m.roughness; d.specular = m.specular; d.pad = 0;
    }
    std::vector<DevQuadLight> lights(desc->n_lights);
    for (uint32_t i = 0; i < desc->n_lights; ++i) {  // DiffuseAreaQuadLight::new, light.rs:61-76
        const pyre_quad_light_desc& l = desc->lights[i];
        DevQuadLight& q = lights[i];
        q.p0 = mk3(l.p0[0], l.p0[1], l.p0[2]);
        q.edge_u = mk3(l.edge_u[0], l.edge_u[1], l.edge_u[2]);
        q.edge_v = mk3(l.edge_v[0], l.edge_v[1], l.edge_v[2]);
        q.emission = mk3(l.emission[0], l.emission[1], l.emission[2]);
        q.crs = cross3(q.edge_u, q.edge_v);
        q.area = len3(q.crs);
        q.inv_cross_len_sq = 1.0f / len2(q.crs);
        q.normal = normalize3(q.crs);
    }

    // ---- environment: texels, CDFs, per-bin pdfs, alias tables (light.rs:214-242)
    EnvTables et;
    DevEnv env{};
    if (desc->env) {
        build_env_tables(desc->env->width, desc->env->height, desc->env->rgb, et);
        env.width = desc->env->width;
        env.height = desc->env->height;
        env.intensity = desc->env->intensity;
    }

    // ---- upload
    DevScene& D = sc->dev;
    std::memset(&D, 0, sizeof D);
    int rc;
    GpuNode* d_nodes = nullptr;
    if (blas.nodes) {  // device-built instance BVHs, then the host-built top levels
        const size_t total = blas.n_nodes + nodes.size();
        cudaError_t e = cudaMalloc(&d_nodes, total * sizeof(GpuNode));
        if (e != cudaSuccess) return fail(cuda_check(ctx, e, "cudaMalloc(scene)"));
        sc->allocations.push_back(d_nodes);
        sc->device_bytes += total * sizeof(GpuNode);
        e = cudaMemcpy(d_nodes, blas.nodes, blas.n_nodes * sizeof(GpuNode), cudaMemcpyDeviceToDevice);
        cudaFree(blas.nodes);
        blas.nodes = nullptr;
        if (e == cudaSuccess && !nodes.empty())
            e = cudaMemcpy(d_nodes + (size_t)node_off, nodes.data(), nodes.size() * sizeof(GpuNode),
                           cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return fail(cuda_check(ctx, e, "cudaMemcpy(scene)"));
    } else if ((rc = upload(ctx, sc, nodes, &d_nodes)) != PYRE_OK) {
        return fail(rc);
    }
    D.nodes = reinterpret_cast<const float4*>(d_nodes);
    float4* d_tris = blas.tris;
    if (!d_tris && (rc = upload(ctx, sc, tris, &d_tris)) != PYRE_OK) return fail(rc);
    D.tris = d_tris;
    DevInstance* d_inst = nullptr;
    if ((rc = upload(ctx, sc, inst, &d_inst)) != PYRE_OK) return fail(rc);
    D.inst = d_inst;
    D.n_inst = (uint32_t)inst.size();
    D.tlas_root = tlas_root;
    uint32_t* d_index = nullptr;
    if ((rc = upload(ctx, sc, index, &d_index)) != PYRE_OK) return fail(rc);
    D.index = d_index;
    float* d_normal = nullptr;
    if ((rc = upload(ctx, sc, normal, &d_normal)) != PYRE_OK) return fail(rc);
    D.normal = d_normal;
    // the vertex normals of each triangle slot (k_slot_normals)
    D.slot_normals = nullptr;
    if (total_tris) {
        std::vector<uint32_t> slot_start, index_base;
        std::vector<uint8_t> has_normals;
        uint32_t acc = 0;
        for (uint32_t m = 0; m < n_meshes; ++m) {
            if (desc->meshes[m].n_triangles == 0) continue;
            slot_start.push_back(acc);
            index_base.push_back((uint32_t)mesh_index_base[m]);
            has_normals.push_back(mesh_normal_base[m] >= 0 ? 1 : 0);
            acc += desc->meshes[m].n_triangles;
        }
        uint32_t *d_start = nullptr, *d_base = nullptr;
        uint8_t* d_has = nullptr;
        if ((rc = upload(ctx, sc, slot_start, &d_start)) != PYRE_OK) return fail(rc);
        if ((rc = upload(ctx, sc, index_base, &d_base)) != PYRE_OK) return fail(rc);
        if ((rc = upload(ctx, sc, has_normals, &d_has)) != PYRE_OK) return fail(rc);
        void* p = nullptr;
        if (injected_alloc_failure(ctx))
            return fail(set_error(ctx, PYRE_ERR_OOM, "cudaMalloc(scene): injected allocation failure"));
        cudaError_t e = cudaMalloc(&p, (size_t)total_tris * 3 * sizeof(float4));
        if (e != cudaSuccess) { cudaGetLastError(); return fail(cuda_check(ctx, e, "cudaMalloc(scene)")); }
        sc->allocations.push_back(p);
        sc->device_bytes += (size_t)total_tris * 3 * sizeof(float4);
        const uint32_t grid = (uint32_t)std::min<uint64_t>((total_tris + 255) / 256, 65535);
        k_slot_normals<<<grid, 256>>>(d_tris, d_index, d_normal, d_start, d_base, d_has, (uint32_t)slot_start.size(),
                                      (uint32_t)total_tris, (float4*)p);
        e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e != cudaSuccess) return fail(cuda_check(ctx, e, "slot normals"));
        D.slot_normals = (const float4*)p;
    }
    DevMaterial* d_mats = nullptr;
    if ((rc = upload(ctx, sc, mats, &d_mats)) != PYRE_OK) return fail(rc);
    D.materials = d_mats;
    D.n_materials = (uint32_t)mats.size();
    DevQuadLight* d_lights = nullptr;
    if ((rc = upload(ctx, sc, lights, &d_lights)) != PYRE_OK) return fail(rc);
    D.lights = d_lights;
    D.n_lights = (uint32_t)lights.size();
    int32_t* d_part_tlas = nullptr;
    uint32_t* d_part_light = nullptr;
    if ((rc = upload(ctx, sc, part_tlas, &d_part_tlas)) != PYRE_OK) return fail(rc);
    if ((rc = upload(ctx, sc, part_light, &d_part_light)) != PYRE_OK) return fail(rc);
    D.part_tlas = d_part_tlas;
    D.part_light = d_part_light;
    D.n_parts = n_parts;
    sc->n_parts = n_parts;
    sc->part_tlas = part_tlas;
    sc->part_light = part_light;
    sc->part_light_max = 0;
    for (uint32_t pp = 0; pp < n_parts; ++pp) sc->part_light_max = std::max(sc->part_light_max, part_light[2 * pp + 1]);
    if (desc->env) {
        float4* px = nullptr;
        float *mc = nullptr, *cc = nullptr, *mp = nullptr, *cp = nullptr;
        float2 *ma = nullptr, *ca = nullptr;
        if ((rc = upload(ctx, sc, et.px, &px)) != PYRE_OK || (rc = upload(ctx, sc, et.marg_cdf, &mc)) != PYRE_OK ||
            (rc = upload(ctx, sc, et.cond_cdf, &cc)) != PYRE_OK || (rc = upload(ctx, sc, et.marg_pdf, &mp)) != PYRE_OK ||
            (rc = upload(ctx, sc, et.cond_pdf, &cp)) != PYRE_OK || (rc = upload(ctx, sc, et.marg_alias, &ma)) != PYRE_OK ||
            (rc = upload(ctx, sc, et.cond_alias, &ca)) != PYRE_OK)
            return fail(rc);
        env.pixels = px; env.marg_cdf = mc; env.cond_cdf = cc; env.marg_pdf = mp; env.cond_pdf = cp;
        env.marg_alias = ma; env.cond_alias = ca;
        D.has_env = 1;
        D.env = env;
    }
    D.error_flag = ctx->d_error;
    sc->n_triangles = (uint32_t)total_tris;
    sc->n_nodes = (uint64_t)node_off + nodes.size();
    *out = sc;
    return PYRE_OK;
}

namespace pyre {

int select_bvh(pyre_ctx* ctx, pyre_scene* scene, uint32_t requested, DevScene* dev, int* width, bool may_build) {
    const uint32_t w = requested ? requested : (uint32_t)scene->bvh_width;
    if (w != 2 && w != 4 && w != 8) return set_error(ctx, PYRE_ERR_INVALID, "bvh_width must be 2, 4 or 8");
    *dev = scene->dev;
    *width = (int)w;
    if (w == 2) return PYRE_OK;
    pyre_scene::Wide& wd = scene->wide[w == 4 ? 0 : 1];
    if (!wd.nodes && scene->dev.n_inst > 0) {
        if (!may_build)
            return set_error(ctx, PYRE_ERR_INVALID, "the scene has no width-" + std::to_string(w) +
                                                        " BVH yet (pyre_scene_set_bvh_width builds it)");
        // collapse from the binary device BVH: one wide BVH per distinct instance BVH
        std::vector<GpuNode> bin(scene->n_nodes);
        std::vector<DevInstance> inst(scene->dev.n_inst);
        PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        PYRE_CUDA_TRY(ctx, cudaMemcpy(bin.data(), scene->dev.nodes, bin.size() * sizeof(GpuNode),
                                      cudaMemcpyDeviceToHost));
        PYRE_CUDA_TRY(ctx, cudaMemcpy(inst.data(), scene->dev.inst, inst.size() * sizeof(DevInstance),
                                      cudaMemcpyDeviceToHost));
        std::vector<float> flat;
        std::map<int32_t, int32_t> wide_of;
        std::vector<int32_t> roots(inst.size(), -1);
        for (size_t k = 0; k < inst.size(); ++k) {
            const int32_t r = inst[k].blas_root;
            if (r < 0) continue;
            auto it = wide_of.find(r);
            if (it == wide_of.end()) it = wide_of.emplace(r, collapse_wide(bin, r, (int)w, flat)).first;
            roots[k] = it->second;
        }
        const uint64_t n_wide = flat.size() / ((size_t)PYRE_WIDE_FIELDS * w);
        if (n_wide * w >= (1ull << 28))
            return set_error(ctx, PYRE_ERR_UNSUPPORTED, "wide BVH too large for its leaf references");
        std::vector<float4> nodes4(flat.size() / 4);
        std::memcpy(nodes4.data(), flat.data(), flat.size() * sizeof(float));
        int rc = upload(ctx, scene, nodes4, &wd.nodes);
        if (!rc) rc = upload(ctx, scene, roots, &wd.root);
        if (rc) { wd.nodes = nullptr; wd.root = nullptr; return rc; }
        wd.n_nodes = n_wide;
    }
    dev->wnodes = wd.nodes;
    dev->wroot = wd.root;
    return PYRE_OK;
}

}  // namespace pyre

extern "C" {

int pyre_scene_upload(pyre_ctx* ctx, const pyre_scene_desc* desc, pyre_scene** out) {
    NvtxRange nvtx("pyre_scene_upload");
    if (!desc) return set_error(ctx, PYRE_ERR_INVALID, "pyre_scene_upload: NULL argument");
    std::vector<uint32_t> inst_part(desc->n_instances, 0), light_part(desc->n_lights, 0);
    return upload_parts(ctx, desc, inst_part, light_part, 1, out);
}

int pyre_scene_upload_batch(pyre_ctx* ctx, const pyre_scene_desc* descs, uint32_t n_parts, pyre_scene** out) {
    NvtxRange nvtx("pyre_scene_upload_batch");
    if (!ctx || !descs || !out || n_parts == 0)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_scene_upload_batch: NULL argument or no parts");
    std::vector<pyre_mesh_desc> meshes;
    std::vector<pyre_instance_desc> insts;
    std::vector<pyre_material_desc> mats;
    std::vector<pyre_quad_light_desc> lights;
    std::vector<uint32_t> inst_part, light_part;
    for (uint32_t p = 0; p < n_parts; ++p) {
        const pyre_scene_desc& d = descs[p];
        if (d.env) return set_error(ctx, PYRE_ERR_UNSUPPORTED, "batched scenes cannot carry environment maps");
        if ((d.n_meshes && !d.meshes) || (d.n_instances && !d.instances) || (d.n_materials && !d.materials) ||
            (d.n_lights && !d.lights))
            return set_error(ctx, PYRE_ERR_INVALID, "batch part " + std::to_string(p) + ": NULL array");
        const uint32_t mesh_base = (uint32_t)meshes.size(), mat_base = (uint32_t)mats.size();
        meshes.insert(meshes.end(), d.meshes, d.meshes + d.n_meshes);
        mats.insert(mats.end(), d.materials, d.materials + d.n_materials);
        for (uint32_t i = 0; i < d.n_instances; ++i) {
            pyre_instance_desc id = d.instances[i];
            if (id.mesh >= d.n_meshes || id.material >= d.n_materials)
                return set_error(ctx, PYRE_ERR_INVALID, "batch part " + std::to_string(p) + ": index out of range");
            id.mesh += mesh_base;
            id.material += mat_base;
            insts.push_back(id);
            inst_part.push_back(p);
        }
        for (uint32_t l = 0; l < d.n_lights; ++l) {
            lights.push_back(d.lights[l]);
            light_part.push_back(p);
        }
    }
    pyre_scene_desc merged;
    std::memset(&merged, 0, sizeof merged);
    merged.meshes = meshes.data(); merged.n_meshes = (uint32_t)meshes.size();
    merged.instances = insts.data(); merged.n_instances = (uint32_t)insts.size();
    merged.materials = mats.data(); merged.n_materials = (uint32_t)mats.size();
    merged.lights = lights.data(); merged.n_lights = (uint32_t)lights.size();
    return upload_parts(ctx, &merged, inst_part, light_part, n_parts, out);
}

int pyre_scene_set_materials(pyre_ctx* ctx, pyre_scene* scene, const pyre_material_desc* materials, uint32_t n) {
    if (!ctx || !scene || (!materials && n)) return set_error(ctx, PYRE_ERR_INVALID, "pyre_scene_set_materials: NULL");
    if (n != scene->dev.n_materials) return set_error(ctx, PYRE_ERR_INVALID, "pyre_scene_set_materials: count differs");
    std::vector<DevMaterial> mats(n);
    for (uint32_t i = 0; i < n; ++i) {
        if (materials[i].kind > PYRE_MAT_DISNEY) return set_error(ctx, PYRE_ERR_INVALID, "unknown material kind");
        DevMaterial& d = mats[i];
        for (int c = 0; c < 3; ++c) d.base[c] = materials[i].base_color[c];
        d.kind = materials[i].kind; d.metallic = materials[i].metallic; d.roughness = materials[i].roughness;
        d.specular = materials[i].specular; d.pad = 0;
    }
    cudaSetDevice(ctx->device);
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (n) PYRE_CUDA_TRY(ctx, cudaMemcpy((void*)scene->dev.materials, mats.data(), n * sizeof(DevMaterial),
                                         cudaMemcpyHostToDevice));
    return PYRE_OK;
}

int pyre_scene_set_env(pyre_ctx* ctx, pyre_scene* scene, const float* rgb, float intensity) {
    if (!ctx || !scene || !rgb) return set_error(ctx, PYRE_ERR_INVALID, "pyre_scene_set_env: NULL argument");
    if (!scene->dev.has_env) return set_error(ctx, PYRE_ERR_INVALID, "pyre_scene_set_env: the scene has no environment");
    DevEnv& E = scene->dev.env;
    EnvTables t;
    build_env_tables(E.width, E.height, rgb, t);
    cudaSetDevice(ctx->device);
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    auto put = [&](const void* dst, const void* src, size_t bytes) {
        return cudaMemcpy(const_cast<void*>(dst), src, bytes, cudaMemcpyHostToDevice);
    };
    cudaError_t e;
    if ((e = put(E.pixels, t.px.data(), t.px.size() * sizeof(float4))) != cudaSuccess ||
        (e = put(E.marg_cdf, t.marg_cdf.data(), t.marg_cdf.size() * 4)) != cudaSuccess ||
        (e = put(E.cond_cdf, t.cond_cdf.data(), t.cond_cdf.size() * 4)) != cudaSuccess ||
        (e = put(E.marg_pdf, t.marg_pdf.data(), t.marg_pdf.size() * 4)) != cudaSuccess ||
        (e = put(E.cond_pdf, t.cond_pdf.data(), t.cond_pdf.size() * 4)) != cudaSuccess ||
        (e = put(E.marg_alias, t.marg_alias.data(), t.marg_alias.size() * sizeof(float2))) != cudaSuccess ||
        (e = put(E.cond_alias, t.cond_alias.data(), t.cond_alias.size() * sizeof(float2))) != cudaSuccess)
        return cuda_check(ctx, e, "pyre_scene_set_env");
    E.intensity = intensity;
    scene->serial = g_scene_serial++;  // cached graphs captured the old intensity
    return PYRE_OK;
}

int pyre_scene_get_info(const pyre_scene* scene, pyre_scene_info* out) {
    if (!scene || !out) return PYRE_ERR_INVALID;
    out->n_triangles = scene->n_triangles;
    out->n_nodes = scene->n_nodes;
    out->n_instances = scene->dev.n_inst;
    out->triangle_bytes = (uint64_t)scene->n_triangles * 48;
    out->node_bytes = scene->n_nodes * 64;
    out->device_bytes = scene->device_bytes;
    return PYRE_OK;
}

int pyre_scene_set_bvh_width(pyre_ctx* ctx, pyre_scene* scene, uint32_t width) {
    if (!ctx || !scene) return set_error(ctx, PYRE_ERR_INVALID, "pyre_scene_set_bvh_width: NULL argument");
    if (width != 2 && width != 4 && width != 8) return set_error(ctx, PYRE_ERR_INVALID, "bvh_width must be 2, 4 or 8");
    cudaSetDevice(ctx->device);
    DevScene dev;
    int w = 2;
    const int rc = select_bvh(ctx, scene, width, &dev, &w);
    if (rc) return rc;
    scene->bvh_width = w;
    return PYRE_OK;
}

int pyre_get_render_stats(const pyre_ctx* ctx, pyre_render_stats* out) {
    if (!ctx || !out) return PYRE_ERR_INVALID;
    *out = ctx->stats;
    return PYRE_OK;
}

int pyre_distribution2d_query(pyre_ctx* ctx, const float* weights, uint32_t width, uint32_t height, int mode,
                              uint32_t n, const float* u, float* samples, uint32_t m, const float* uv, float* pdfs) {
    if (!ctx || !weights || width == 0 || height == 0 || (n && (!u || !samples)) || (m && (!uv || !pdfs)))
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_distribution2d_query: bad arguments");
    cudaSetDevice(ctx->device);
    EnvTables t;
    build_dist2d(width, height, weights, t);
    const size_t bytes[] = {t.marg_cdf.size() * 4, t.cond_cdf.size() * 4, t.marg_pdf.size() * 4, t.cond_pdf.size() * 4,
                            t.marg_alias.size() * 8, t.cond_alias.size() * 8, (size_t)n * 8, (size_t)n * 20,
                            (size_t)m * 8, (size_t)m * 4};
    size_t off[11] = {0};
    for (int k = 0; k < 10; ++k) off[k + 1] = off[k] + ((bytes[k] + 255) & ~(size_t)255);
    int rc = ensure_workspace(ctx, ctx->io_ws, off[10] + 256);
    if (rc) return rc;
    char* b = (char*)ctx->io_ws.ptr;
    cudaStream_t st = ctx->stream;
    const void* src[] = {t.marg_cdf.data(), t.cond_cdf.data(), t.marg_pdf.data(), t.cond_pdf.data(),
                         t.marg_alias.data(), t.cond_alias.data(), u, nullptr, uv, nullptr};
    for (int k = 0; k < 10; ++k)
        if (src[k] && bytes[k]) PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(b + off[k], src[k], bytes[k], cudaMemcpyHostToDevice, st));
    DevEnv E{};
    E.width = width; E.height = height; E.intensity = 1.0f;
    E.marg_cdf = (const float*)(b + off[0]); E.cond_cdf = (const float*)(b + off[1]);
    E.marg_pdf = (const float*)(b + off[2]); E.cond_pdf = (const float*)(b + off[3]);
    E.marg_alias = (const float2*)(b + off[4]); E.cond_alias = (const float2*)(b + off[5]);
    const uint32_t threads = std::max(n, m);
    if (threads)
        k_dist2d_query<<<(threads + 255) / 256, 256, 0, st>>>(E, mode == PYRE_ENV_CDF ? 1 : 0, (const float*)(b + off[6]), n,
                                                              (const float*)(b + off[8]), m, (float*)(b + off[7]),
                                                              (float*)(b + off[9]));
    PYRE_CUDA_TRY(ctx, cudaGetLastError());
    if (n) PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(samples, b + off[7], bytes[7], cudaMemcpyDeviceToHost, st));
    if (m) PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(pdfs, b + off[9], bytes[9], cudaMemcpyDeviceToHost, st));
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return PYRE_OK;
}

int pyre_bsdf_query(pyre_ctx* ctx, const pyre_material_desc* mat, uint32_t n, const float* wo, const float* u,
                    float* out) {
    if (!ctx || !mat || (n && (!wo || !u || !out)) || mat->kind > PYRE_MAT_DISNEY)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_bsdf_query: bad arguments");
    if (n == 0) return PYRE_OK;
    cudaSetDevice(ctx->device);
    const size_t b_wo = ((size_t)n * 12 + 255) & ~(size_t)255, b_u = ((size_t)n * 8 + 255) & ~(size_t)255;
    int rc = ensure_workspace(ctx, ctx->io_ws, b_wo + b_u + (size_t)n * 52 + 256);
    if (rc) return rc;
    char* b = (char*)ctx->io_ws.ptr;
    cudaStream_t st = ctx->stream;
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(b, wo, (size_t)n * 12, cudaMemcpyHostToDevice, st));
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(b + b_wo, u, (size_t)n * 8, cudaMemcpyHostToDevice, st));
    Bsdf bs;
    bs.kind = mat->kind;
    bs.base = mk3(mat->base_color[0], mat->base_color[1], mat->base_color[2]);
    bs.metallic = mat->metallic; bs.roughness = mat->roughness; bs.specular = mat->specular;
    k_bsdf_query<<<(n + 255) / 256, 256, 0, st>>>(bs, (const float*)b, (const float*)(b + b_wo), n,
                                                   (float*)(b + b_wo + b_u));
    PYRE_CUDA_TRY(ctx, cudaGetLastError());
    PYRE_CUDA_TRY(ctx, cudaMemcpyAsync(out, b + b_wo + b_u, (size_t)n * 52, cudaMemcpyDeviceToHost, st));
    PYRE_CUDA_TRY(ctx, cudaStreamSynchronize(st));
    return PYRE_OK;
}

int pyre_inject_alloc_failure(pyre_ctx* ctx, int after) {
    if (!ctx) return PYRE_ERR_INVALID;
    ctx->fail_alloc_countdown = after < 0 ? -1 : after;
    return PYRE_OK;
}

int pyre_set_bvh_builder(pyre_ctx* ctx, int builder) {
    if (!ctx) return PYRE_ERR_INVALID;
    if (builder != PYRE_BVH_BUILDER_HOST && builder != PYRE_BVH_BUILDER_DEVICE)
        return set_error(ctx, PYRE_ERR_INVALID, "unknown BVH builder");
    ctx->bvh_builder = builder;
    return PYRE_OK;
}

int pyre_set_stage_timing(pyre_ctx* ctx, int enabled) {
    if (!ctx) return PYRE_ERR_INVALID;
    ctx->stage_timing = enabled ? 1 : 0;
    return PYRE_OK;
}

}  // extern "C"
