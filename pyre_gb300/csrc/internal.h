// internal.h — context and scene objects behind the C ABI.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include <string>
#include <vector>
#include "../../include/pyre_cuda.h"
#include "bvh_host.h"
#include "device_scene.cuh"

struct pyre_scene {
    pyre::DevScene dev;
    uint64_t serial = 0;  // unique per upload; keys cached CUDA graphs
    std::vector<void*> allocations;  // device buffers owned by the scene
    std::vector<int32_t> slot_of_instance;  // original instance id -> device slot
    uint32_t n_triangles = 0;
    uint64_t n_nodes = 0;
    uint32_t n_parts = 1;         // sub-scenes (pyre_scene_upload_batch)
    uint32_t part_light_max = 0;  // most quad lights in one part
    std::vector<int32_t> part_tlas;    // host copies of the per-part tables
    std::vector<uint32_t> part_light;  // (first, count) per part
    uint64_t device_bytes = 0;
    // wide BVHs built on first use (index 0: width 4, 1: width 8)
    struct Wide {
        float4* nodes = nullptr;
        int32_t* root = nullptr;  // per instance slot
        uint64_t n_nodes = 0;
    } wide[2];
    int bvh_width = 2;  // traversal width when a call does not choose one
};

// Reusable device workspace of a context (grown on demand, freed at destroy).
struct Workspace {
    void* ptr = nullptr;
    size_t bytes = 0;
};

struct pyre_ctx {
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    std::string error;
    int* d_error = nullptr;     // kernel-reported status (PYRE_ERR_OVERFLOW ...)
    unsigned int* d_counter = nullptr;  // work counter of the intersect kernels
    Workspace render_ws;        // path state of the wavefront integrator
    Workspace io_ws;            // staging for host-memory rays / films
    Workspace tape_ws;          // pyre_forward: per-path radiance for pyre_backward
    Workspace prog_ws;          // pyre_render_progressive: device copy of a host running mean
    int bvh_builder = PYRE_BVH_BUILDER_HOST;  // where pyre_scene_upload builds instance BVHs
    int64_t fail_alloc_countdown = -1;  // pyre_inject_alloc_failure: allocations until one fails
    std::string tape_key;       // the render that tape_ws holds
    pyre_render_stats stats{};
    int stage_timing = 0;
    cudaEvent_t ev[16] = {};
    // Stage timing: one event between consecutive stage kernels, with the
    // stage (0 extend, 1 shade, 2 shadow, 3 other) of the kernel that follows.
    std::vector<cudaEvent_t> stage_ev;
    std::vector<int> stage_tag;
    size_t stage_used = 0;
    // CUDA graph of one wave, keyed by the render configuration it was captured for.
    cudaGraphExec_t wave_graph = nullptr;
    std::string wave_graph_key;
    // pyre_render_batch: films of finished jobs are copied on this stream while later waves render; one
    // event per wave marks the jobs it completes
    cudaStream_t copy_stream = nullptr;
    std::vector<cudaEvent_t> wave_ev;
};

namespace pyre {
int set_error(pyre_ctx* ctx, int code, const std::string& msg);
int cuda_check(pyre_ctx* ctx, cudaError_t e, const char* what);
// Grows `ws` to at least `bytes` (contents not preserved).
int ensure_workspace(pyre_ctx* ctx, Workspace& ws, size_t bytes);
// True (once) when an injected allocation failure is due (pyre_inject_alloc_failure).
bool injected_alloc_failure(pyre_ctx* ctx);
// Reads and clears the kernel error flag; returns its status.
int take_kernel_error(pyre_ctx* ctx);
// The scene as the traversal kernels of one call see it: `requested` width
// (0 = the scene's default) is checked, its wide BVH built if needed, and
// `dev` gets a copy of the scene with the wide arrays set; *width = 2, 4, 8.
// With may_build false a wide BVH that does not exist yet is an error.
int select_bvh(pyre_ctx* ctx, pyre_scene* scene, uint32_t requested, DevScene* dev, int* width,
               bool may_build = true);
// Builds the reference BVH of meshes `mesh_ids` (all with triangles, in
// this order: their triangle slots follow one another) on the GPU and lays
// out their device nodes and triangle records (bvh_device.cu).
int device_build_blas(pyre_ctx* ctx, const pyre_scene_desc* desc, const std::vector<uint32_t>& mesh_ids,
                      DeviceBlas* out);
}  // namespace pyre

// An NVTX range over one public call (visible in nsys / ncu timelines; free
// when no tool is attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

#define PYRE_CUDA_TRY(ctx, expr)                                   \
    do {                                                           \
        cudaError_t _e = (expr);                                   \
        if (_e != cudaSuccess) return pyre::cuda_check(ctx, _e, #expr); \
    } while (0)
