// bvh_device.cu — the reference's SAH-binned BVH build on the GPU.
//
// Produces, for each mesh, the same node array and primitive order as
// Bvh::build (crates/pyre/src/geometry/bvh.rs:45-64,180-409; restated on the
// host in bvh_host.cpp): 12 bins on the longest centroid axis, cost
// 1 + 2 (nL AL + nR AR) / A, leaves of at most 8 primitives, the midpoint and
// equal-count fallbacks, depth-first pre-order with the left child next.
//
// The recursion becomes a breadth-first loop over levels; every level
// processes all open tasks (node ranges) of all meshes at once:
//   box      primitive and centroid bounds per task (warp-segmented
//            reductions, then order-preserving integer atomics: min and max
//            are exact, so the result does not depend on the order)
//   prepare  single-primitive and coincident-centroid leaves, bin setup
//   bin      12-bin counts and boxes per task
//   decide   the prefix/suffix sweeps and SAH costs in the reference's order,
//            leaf or partition position
//   flags / scan / tables / scatter
//            the reference's in-place partition (two pointers, swap from the
//            end) computed in parallel from its closed form: with mid the
//            number of primitives left of the split, the k-th right-side
//            primitive of [start, mid) moves to l(k-1) - 1 and the k-th
//            left-side primitive of [mid, end) counted from the end (at l(k))
//            takes its place (l(0) = end); a right-side primitive at mid moves
//            to l(K) - 1 (K such pairs); any other right-side primitive at
//            q >= mid moves to q - 1
//   finish   node records, the equal-count fallback, the next level's tasks
// Node ids are breadth-first; sizes of subtrees (bottom-up) then give each
// node its depth-first index (top-down), and the emit kernels write the
// reference layout or the 64-byte device nodes directly.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "bvh_host.h"
#include "internal.h"

namespace pyre {
namespace {

constexpr int kBins = 12;
constexpr uint32_t kMaxLeaf = 8;
constexpr int kScanBlock = 1024;  // threads of the scan kernels, 4 elements each
enum : int { MODE_LEAF = 0, MODE_BIN = 1, MODE_PART = 2, MODE_SPLIT = 3 };

// float <-> unsigned with the same order (for atomicMin / atomicMax)
__device__ __forceinline__ uint32_t ord(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unord(uint32_t o) {
    return __uint_as_float((o & 0x80000000u) ? (o & 0x7fffffffu) : ~o);
}
__device__ __forceinline__ float comp4(float4 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
__device__ __forceinline__ int32_t to_i32(float f) {  // Rust `as i32`
    if (f != f) return 0;
    if (f >= 2147483647.0f) return 2147483647;
    if (f <= -2147483648.0f) return (int32_t)0x80000000;
    return (int32_t)f;
}

struct Task {
    uint32_t start, end;  // positions in the primitive order
    uint32_t node;        // breadth-first node id
    uint32_t mesh;
};

struct TaskAcc {
    uint32_t lo[3], hi[3], clo[3], chi[3];
    uint32_t bin_n[kBins];
    uint32_t bin_lo[kBins][3], bin_hi[kBins][3];
};

struct TaskState {
    int mode, axis;
    float cmin, scale, extent, split;
    uint32_t mid;                  // first position of the right child
    uint32_t left_task, right_task;
    uint32_t leaf_count;
};

struct BNode {
    float lo[3], hi[3];
    uint32_t start, count;   // leaf: positions [start, start + count)
    int32_t left, right;     // interior: breadth-first children; -1 for a leaf
    uint32_t axis, mesh;
};

__device__ __forceinline__ float area(float lx, float ly, float lz, float hx, float hy, float hz) {
    const float dx = hx - lx, dy = hy - ly, dz = hz - lz;
    return 2.0f * (dx * dy + dx * dz + dy * dz);
}

// Per-triangle bounds and centroid (mesh.rs:32-40, as triangle_bounds).
__global__ void k_tri_bounds(const float* __restrict__ pos, const uint32_t* __restrict__ idx, uint32_t n,
                             float4* blo, float4* bhi, float4* cen) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        const uint32_t i0 = idx[3 * (size_t)t], i1 = idx[3 * (size_t)t + 1], i2 = idx[3 * (size_t)t + 2];
        const f3 a = mk3(pos[3 * (size_t)i0], pos[3 * (size_t)i0 + 1], pos[3 * (size_t)i0 + 2]);
        const f3 b = mk3(pos[3 * (size_t)i1], pos[3 * (size_t)i1 + 1], pos[3 * (size_t)i1 + 2]);
        const f3 c = mk3(pos[3 * (size_t)i2], pos[3 * (size_t)i2 + 1], pos[3 * (size_t)i2 + 2]);
        const f3 lo = vmin3(vmin3(a, b), c), hi = vmax3(vmax3(a, b), c);
        const f3 m = (a + b + c) / 3.0f;
        blo[t] = make_float4(lo.x, lo.y, lo.z, 0.0f);
        bhi[t] = make_float4(hi.x, hi.y, hi.z, 0.0f);
        cen[t] = make_float4(m.x, m.y, m.z, 0.0f);
    }
}

__global__ void k_init_acc(TaskAcc* acc, uint32_t n_tasks) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tasks) return;
    TaskAcc& a = acc[t];
    const uint32_t lo = 0xFF800000u /* ord(+inf) */, hi = 0x007FFFFFu /* ord(-inf) */;
    for (int k = 0; k < 3; ++k) { a.lo[k] = lo; a.hi[k] = hi; a.clo[k] = lo; a.chi[k] = hi; }
    for (int b = 0; b < kBins; ++b) {
        a.bin_n[b] = 0;
        for (int k = 0; k < 3; ++k) { a.bin_lo[b][k] = lo; a.bin_hi[b][k] = hi; }
    }
}

// Reduces v over the lanes of `peers` and lets its first lane apply the atomic.
__device__ __forceinline__ void seg_min(unsigned peers, bool leader, uint32_t* dst, uint32_t v) {
    v = __reduce_min_sync(peers, v);
    if (leader) atomicMin(dst, v);
}
__device__ __forceinline__ void seg_max(unsigned peers, bool leader, uint32_t* dst, uint32_t v) {
    v = __reduce_max_sync(peers, v);
    if (leader) atomicMax(dst, v);
}

// Grid-stride loops over positions run whole warps per round (every lane
// of a warp takes part in the warp-collective operations of each round).
#define WARP_ROUNDS(wb, n)                                                                            \
    for (uint32_t wb = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); wb < (n); wb += gridDim.x * blockDim.x)

__global__ void k_box(const int32_t* __restrict__ pos_task, const uint32_t* __restrict__ idx,
                      const float4* __restrict__ blo, const float4* __restrict__ bhi,
                      const float4* __restrict__ cen, uint32_t n, TaskAcc* acc) {
    const int lane = threadIdx.x & 31;
    WARP_ROUNDS(wb, n) {
        const uint32_t p = wb + lane;
        const int32_t t = p < n ? pos_task[p] : -1;
        const unsigned peers = __match_any_sync(0xffffffffu, t);
        if (t < 0) continue;
        const bool leader = lane == __ffs(peers) - 1;
        const uint32_t prim = idx[p];
        const float4 lo = blo[prim], hi = bhi[prim], c = cen[prim];
        TaskAcc& a = acc[t];
        seg_min(peers, leader, &a.lo[0], ord(lo.x)); seg_min(peers, leader, &a.lo[1], ord(lo.y));
        seg_min(peers, leader, &a.lo[2], ord(lo.z));
        seg_max(peers, leader, &a.hi[0], ord(hi.x)); seg_max(peers, leader, &a.hi[1], ord(hi.y));
        seg_max(peers, leader, &a.hi[2], ord(hi.z));
        seg_min(peers, leader, &a.clo[0], ord(c.x)); seg_min(peers, leader, &a.clo[1], ord(c.y));
        seg_min(peers, leader, &a.clo[2], ord(c.z));
        seg_max(peers, leader, &a.chi[0], ord(c.x)); seg_max(peers, leader, &a.chi[1], ord(c.y));
        seg_max(peers, leader, &a.chi[2], ord(c.z));
    }
}

// bvh.rs:189-211: leaves of one primitive or of coincident centroids; bins otherwise.
__global__ void k_prepare(const Task* __restrict__ tasks, const TaskAcc* __restrict__ acc, uint32_t n_tasks,
                          TaskState* st) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tasks) return;
    const Task T = tasks[t];
    const TaskAcc& a = acc[t];
    TaskState s{};
    const uint32_t n = T.end - T.start;
    const float dx = unord(a.chi[0]) - unord(a.clo[0]), dy = unord(a.chi[1]) - unord(a.clo[1]),
                dz = unord(a.chi[2]) - unord(a.clo[2]);
    const int axis = (dx >= dy && dx >= dz) ? 0 : (dy >= dz ? 1 : 2);
    const float extent = axis == 0 ? dx : (axis == 1 ? dy : dz);
    if (n == 1) {
        s.mode = MODE_LEAF; s.leaf_count = 1;
    } else if (extent < 1e-9f) {
        s.mode = MODE_LEAF; s.leaf_count = min(n, 65535u);
    } else {
        s.mode = MODE_BIN;
        s.axis = axis;
        s.extent = extent;
        s.cmin = unord(a.clo[axis]);
        s.scale = (float)kBins / extent;
    }
    st[t] = s;
}

__global__ void k_bin(const int32_t* __restrict__ pos_task, const uint32_t* __restrict__ idx,
                      const float4* __restrict__ blo, const float4* __restrict__ bhi,
                      const float4* __restrict__ cen, uint32_t n, const TaskState* __restrict__ st, TaskAcc* acc) {
    const int lane = threadIdx.x & 31;
    WARP_ROUNDS(wb, n) {
        const uint32_t p = wb + lane;
        int32_t t = p < n ? pos_task[p] : -1;
        int b = 0;
        uint32_t prim = 0;
        if (t >= 0) {
            const TaskState& s = st[t];
            if (s.mode != MODE_BIN) t = -1;
            else {
                prim = idx[p];
                b = to_i32((comp4(cen[prim], s.axis) - s.cmin) * s.scale);
                b = min(max(b, 0), kBins - 1);
            }
        }
        const long long key = t < 0 ? -1ll : (long long)t * kBins + b;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (t < 0) continue;
        const bool leader = lane == __ffs(peers) - 1;
        TaskAcc& a = acc[t];
        if (leader) atomicAdd(&a.bin_n[b], (uint32_t)__popc(peers));
        const float4 lo = blo[prim], hi = bhi[prim];
        seg_min(peers, leader, &a.bin_lo[b][0], ord(lo.x)); seg_min(peers, leader, &a.bin_lo[b][1], ord(lo.y));
        seg_min(peers, leader, &a.bin_lo[b][2], ord(lo.z));
        seg_max(peers, leader, &a.bin_hi[b][0], ord(hi.x)); seg_max(peers, leader, &a.bin_hi[b][1], ord(hi.y));
        seg_max(peers, leader, &a.bin_hi[b][2], ord(hi.z));
    }
}

// bvh.rs:236-321: sweeps, costs, leaf test, partition position.
__global__ void k_decide(const Task* __restrict__ tasks, const TaskAcc* __restrict__ acc, uint32_t n_tasks,
                         TaskState* st) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tasks) return;
    TaskState s = st[t];
    if (s.mode != MODE_BIN) return;
    const Task T = tasks[t];
    const TaskAcc& a = acc[t];
    const uint32_t n = T.end - T.start;
    uint32_t ln[kBins - 1], rn[kBins - 1];
    float la[kBins - 1], ra[kBins - 1];
    {
        uint32_t c = 0;
        float lx = INFINITY, ly = INFINITY, lz = INFINITY, hx = -INFINITY, hy = -INFINITY, hz = -INFINITY;
        for (int i = 0; i < kBins - 1; ++i) {
            c += a.bin_n[i];
            lx = fminf(lx, unord(a.bin_lo[i][0])); ly = fminf(ly, unord(a.bin_lo[i][1]));
            lz = fminf(lz, unord(a.bin_lo[i][2]));
            hx = fmaxf(hx, unord(a.bin_hi[i][0])); hy = fmaxf(hy, unord(a.bin_hi[i][1]));
            hz = fmaxf(hz, unord(a.bin_hi[i][2]));
            ln[i] = c;
            la[i] = area(lx, ly, lz, hx, hy, hz);
        }
        c = 0;
        lx = ly = lz = INFINITY; hx = hy = hz = -INFINITY;
        for (int i = kBins - 2; i >= 0; --i) {
            c += a.bin_n[i + 1];
            lx = fminf(lx, unord(a.bin_lo[i + 1][0])); ly = fminf(ly, unord(a.bin_lo[i + 1][1]));
            lz = fminf(lz, unord(a.bin_lo[i + 1][2]));
            hx = fmaxf(hx, unord(a.bin_hi[i + 1][0])); hy = fmaxf(hy, unord(a.bin_hi[i + 1][1]));
            hz = fmaxf(hz, unord(a.bin_hi[i + 1][2]));
            rn[i] = c;
            ra[i] = area(lx, ly, lz, hx, hy, hz);
        }
    }
    const float parent_area = fmaxf(area(unord(a.lo[0]), unord(a.lo[1]), unord(a.lo[2]), unord(a.hi[0]),
                                         unord(a.hi[1]), unord(a.hi[2])),
                                    1e-9f);
    float best = INFINITY;
    int best_i = 0;
    for (int i = 0; i < kBins - 1; ++i) {
        if (ln[i] == 0 || rn[i] == 0) continue;
        const float cost = 1.0f + 2.0f * ((float)ln[i] * la[i] + (float)rn[i] * ra[i]) / parent_area;
        if (cost < best) { best = cost; best_i = i; }
    }
    if (!isfinite(best)) {
        s.mode = MODE_PART;
        s.split = s.cmin + 0.5f * s.extent;
    } else if (n <= kMaxLeaf && best >= 2.0f * (float)n) {
        s.mode = MODE_LEAF;
        s.leaf_count = n;
    } else {
        s.mode = MODE_PART;
        s.split = s.cmin + (float)(best_i + 1) * s.extent / (float)kBins;
    }
    st[t] = s;
}

__global__ void k_flags(const int32_t* __restrict__ pos_task, const uint32_t* __restrict__ idx,
                        const float4* __restrict__ cen, uint32_t n, const TaskState* __restrict__ st,
                        uint32_t* flag) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int32_t t = pos_task[p];
        uint32_t f = 0;
        if (t >= 0) {
            const TaskState& s = st[t];
            if (s.mode == MODE_PART) f = comp4(cen[idx[p]], s.axis) < s.split ? 1u : 0u;
        }
        flag[p] = f;
    }
}

// Exclusive scan of flag[0, n) into pre[0, n] (pre[n] = total): block scans
// of 4 * kScanBlock elements, a scan of the block sums, then the offsets.
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* warp_tot, uint32_t* total) {
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_tot[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < (blockDim.x >> 5) ? warp_tot[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= (uint32_t)o) w += y;
        }
        warp_tot[lane] = w;
    }
    __syncthreads();
    const uint32_t r = (warp ? warp_tot[warp - 1] : 0u) + x - v;
    if (total) *total = warp_tot[(blockDim.x >> 5) - 1];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_local(const uint32_t* __restrict__ in, uint32_t n,
                                                           uint32_t* out, uint32_t* block_sum) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t tot;
    const uint64_t base = (uint64_t)blockIdx.x * 4 * kScanBlock + 4 * (uint64_t)threadIdx.x;
    uint32_t v[4], s = 0;
    for (int k = 0; k < 4; ++k) { v[k] = base + k < n ? in[base + k] : 0u; s += v[k]; }
    uint32_t off = block_excl_scan(s, warp_tot, threadIdx.x == 0 ? &tot : nullptr);
    __syncthreads();
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) out[base + k] = off;
        off += v[k];
    }
    if (threadIdx.x == 0) block_sum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kScanBlock) k_scan_sums(uint32_t* block_sum, uint32_t n_blocks, uint32_t* total) {
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t tot;
    uint32_t carry = 0;
    for (uint32_t b0 = 0; b0 < n_blocks; b0 += kScanBlock) {
        const uint32_t i = b0 + threadIdx.x;
        const uint32_t v = i < n_blocks ? block_sum[i] : 0u;
        const uint32_t e = block_excl_scan(v, warp_tot, threadIdx.x == 0 ? &tot : nullptr);
        __syncthreads();
        if (i < n_blocks) block_sum[i] = carry + e;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void k_scan_add(uint32_t* out, uint32_t n, const uint32_t* __restrict__ block_sum,
                           const uint32_t* __restrict__ total) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p <= n; p += gridDim.x * blockDim.x) {
        if (p == n) out[n] = *total;
        else out[p] += block_sum[p / (4 * kScanBlock)];
    }
}

// Rank tables of the partition: front[start + k - 1] = position of the k-th
// right-side primitive of [start, mid); back[start + r - 1] = position of the
// r-th left-side primitive of [mid, end) counted from the end.
__global__ void k_tables(const int32_t* __restrict__ pos_task, const Task* __restrict__ tasks,
                         const TaskState* __restrict__ st, const uint32_t* __restrict__ flag,
                         const uint32_t* __restrict__ pre, uint32_t n, uint32_t* front, uint32_t* back) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int32_t t = pos_task[p];
        if (t < 0 || st[t].mode != MODE_PART) continue;
        const Task T = tasks[t];
        const uint32_t Lb = pre[p] - pre[T.start], Lt = pre[T.end] - pre[T.start];
        const uint32_t mid = T.start + Lt;
        if (p < mid) {
            if (!flag[p]) front[T.start + (p - T.start - Lb)] = p;
        } else if (flag[p]) {
            back[T.start + (Lt - Lb) - 1] = p;
        }
    }
}

__global__ void k_scatter(const int32_t* __restrict__ pos_task, const Task* __restrict__ tasks,
                          const TaskState* __restrict__ st, const uint32_t* __restrict__ flag,
                          const uint32_t* __restrict__ pre, const uint32_t* __restrict__ front,
                          const uint32_t* __restrict__ back, const uint32_t* __restrict__ idx, uint32_t n,
                          uint32_t* idx_next) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int32_t t = pos_task[p];
        uint32_t dst = p;
        if (t >= 0 && st[t].mode == MODE_PART) {
            const Task T = tasks[t];
            const uint32_t Lb = pre[p] - pre[T.start], Lt = pre[T.end] - pre[T.start];
            const uint32_t mid = T.start + Lt;
            const uint32_t K = (mid - T.start) - (pre[mid] - pre[T.start]);  // right-side primitives left of mid
            auto l_of = [&](uint32_t k) { return k == 0 ? T.end : back[T.start + k - 1]; };
            if (p < mid) {
                if (!flag[p]) dst = l_of(p - T.start - Lb) - 1;  // k-th: l(k - 1) - 1
            } else if (flag[p]) {
                dst = front[T.start + (Lt - Lb) - 1];
            } else {
                dst = p == mid ? l_of(K) - 1 : p - 1;
            }
        }
        idx_next[dst] = idx[p];
    }
}

// Node records and the next level's tasks.
__global__ void k_finish(const Task* __restrict__ tasks, const TaskAcc* __restrict__ acc, uint32_t n_tasks,
                         const uint32_t* __restrict__ pre, TaskState* st, BNode* nodes, Task* next,
                         uint32_t* counters /* [0] next tasks, [1] nodes */) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_tasks) return;
    const Task T = tasks[t];
    TaskState s = st[t];
    const TaskAcc& a = acc[t];
    const uint32_t n = T.end - T.start;
    BNode nd;
    for (int k = 0; k < 3; ++k) { nd.lo[k] = unord(a.lo[k]); nd.hi[k] = unord(a.hi[k]); }
    nd.mesh = T.mesh;
    uint32_t mid = 0;
    if (s.mode == MODE_PART) {
        mid = T.start + (pre[T.end] - pre[T.start]);
        if (mid == T.start || mid == T.end) {
            if (n <= kMaxLeaf) { s.mode = MODE_LEAF; s.leaf_count = n; }
            else mid = T.start + n / 2;
        }
    }
    if (s.mode == MODE_LEAF) {
        nd.start = T.start; nd.count = s.leaf_count; nd.left = nd.right = -1; nd.axis = 0;
    } else {
        s.mode = MODE_SPLIT;
        s.mid = mid;
        const uint32_t nt = atomicAdd(&counters[0], 2u), nn = atomicAdd(&counters[1], 2u);
        s.left_task = nt; s.right_task = nt + 1;
        next[nt] = Task{T.start, mid, nn, T.mesh};
        next[nt + 1] = Task{mid, T.end, nn + 1, T.mesh};
        nd.start = 0; nd.count = 0; nd.left = (int32_t)nn; nd.right = (int32_t)nn + 1; nd.axis = (uint32_t)s.axis;
    }
    nodes[T.node] = nd;
    st[t] = s;
}

__global__ void k_assign(int32_t* pos_task, const TaskState* __restrict__ st, uint32_t n) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const int32_t t = pos_task[p];
        if (t < 0) continue;
        const TaskState& s = st[t];
        pos_task[p] = s.mode != MODE_SPLIT ? -1 : (int32_t)(p < s.mid ? s.left_task : s.right_task);
    }
}

// Subtree sizes (all nodes / interior nodes), one breadth-first level.
__global__ void k_sizes(const BNode* __restrict__ nodes, uint32_t first, uint32_t count, uint32_t* size,
                        uint32_t* isize) {
    const uint32_t v = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= first + count) return;
    const BNode& nd = nodes[v];
    if (nd.left < 0) { size[v] = 1; isize[v] = 0; return; }
    size[v] = 1 + size[nd.left] + size[nd.right];
    isize[v] = 1 + isize[nd.left] + isize[nd.right];
}

// Depth-first index of every node and of every interior node, one level.
__global__ void k_order(const BNode* __restrict__ nodes, uint32_t first, uint32_t count,
                        const uint32_t* __restrict__ size, const uint32_t* __restrict__ isize, uint32_t* dfs,
                        uint32_t* ifs) {
    const uint32_t v = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= first + count) return;
    const BNode& nd = nodes[v];
    if (nd.left < 0) return;
    dfs[nd.left] = dfs[v] + 1;
    dfs[nd.right] = dfs[v] + 1 + size[nd.left];
    ifs[nd.left] = ifs[v] + 1;
    ifs[nd.right] = ifs[v] + 1 + isize[nd.left];
}

// The reference layout of every node (pyre_bvh2_node) into its mesh's range.
__global__ void k_emit_ref(const BNode* __restrict__ nodes, uint32_t n_nodes, const uint32_t* __restrict__ dfs,
                           const uint32_t* __restrict__ mesh_node_base, const uint32_t* __restrict__ mesh_prim_base,
                           pyre_bvh2_node* out) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_nodes) return;
    const BNode& nd = nodes[v];
    pyre_bvh2_node r;
    for (int k = 0; k < 3; ++k) { r.bounds_min[k] = nd.lo[k]; r.bounds_max[k] = nd.hi[k]; }
    if (nd.left < 0) {
        r.offset = nd.start - mesh_prim_base[nd.mesh];
        r.n_primitives = (uint16_t)nd.count;
        r.axis = 0;
    } else {
        r.offset = dfs[nd.right];
        r.n_primitives = 0;
        r.axis = (uint8_t)nd.axis;
    }
    r.pad = 0;
    out[mesh_node_base[nd.mesh] + dfs[v]] = r;
}

__global__ void k_emit_prims(const uint32_t* __restrict__ idx, uint32_t n, const uint32_t* __restrict__ prim_mesh,
                             const uint32_t* __restrict__ mesh_prim_base, uint32_t* out) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        out[p] = idx[p] - mesh_prim_base[prim_mesh[p]];
}

__global__ void k_prim_mesh(const uint32_t* __restrict__ mesh_prim_base, uint32_t n_meshes, uint32_t n,
                            uint32_t* prim_mesh, int32_t* pos_task, uint32_t* idx) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = n_meshes - 1;  // last mesh whose base is <= p
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) / 2;
            if (mesh_prim_base[mid] <= p) lo = mid; else hi = mid - 1;
        }
        prim_mesh[p] = lo;
        pos_task[p] = (int32_t)lo;  // level 0: task m = mesh m
        idx[p] = p;
    }
}

// 64-byte device nodes (GpuNode, bvh_host.h) of every mesh: interior node v
// of mesh m becomes node node_base[m] + ifs[v]; a mesh whose root is a leaf
// gets one node holding that leaf and an empty slot, as collapse_bvh2 does.
// Leaf children point at triangle slots, which are the build's positions.
__global__ void k_emit_gpu(const BNode* __restrict__ nodes, uint32_t n_nodes, uint32_t n_meshes,
                           const uint32_t* __restrict__ ifs, const uint32_t* __restrict__ node_base, GpuNode* out) {
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n_nodes) return;
    const BNode& nd = nodes[v];
    const bool root = v < n_meshes;
    if (nd.left < 0 && !root) return;
    GpuNode g;
    auto put = [&](int s, const BNode& c) {
        float* xy = s == 0 ? g.a : g.b;
        xy[0] = c.lo[0]; xy[1] = c.hi[0]; xy[2] = c.lo[1]; xy[3] = c.hi[1];
        g.c[2 * s] = c.lo[2]; g.c[2 * s + 1] = c.hi[2];
    };
    if (nd.left < 0) {  // a root leaf
        put(0, nd);
        g.d[0] = (int32_t)nd.start; g.d[2] = (int32_t)nd.count;
        g.b[0] = INFINITY; g.b[1] = -INFINITY; g.b[2] = INFINITY; g.b[3] = -INFINITY;
        g.c[2] = INFINITY; g.c[3] = -INFINITY;
        g.d[1] = -1; g.d[3] = 0;
        out[node_base[nd.mesh]] = g;
        return;
    }
    const int32_t kid[2] = {nd.left, nd.right};
    for (int s = 0; s < 2; ++s) {
        const BNode& c = nodes[kid[s]];
        put(s, c);
        if (c.left < 0) { g.d[s] = (int32_t)c.start; g.d[2 + s] = (int32_t)c.count; }
        else { g.d[s] = (int32_t)(node_base[nd.mesh] + ifs[kid[s]]); g.d[2 + s] = 0; }
    }
    out[node_base[nd.mesh] + ifs[v]] = g;
}

// Triangle records in slot (= build position) order: (v0, local triangle id),
// e1 = v1 - v0, e2 = v2 - v0 (as pyre_scene_upload lays them out).
__global__ void k_emit_tris(const uint32_t* __restrict__ idx, uint32_t n, const uint32_t* __restrict__ prim_mesh,
                            const uint32_t* __restrict__ mesh_prim_base, const float* __restrict__ pos,
                            const uint32_t* __restrict__ vidx, float4* tris) {
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const uint32_t t = idx[p];
        const uint32_t local = t - mesh_prim_base[prim_mesh[p]];
        const uint32_t i0 = vidx[3 * (size_t)t], i1 = vidx[3 * (size_t)t + 1], i2 = vidx[3 * (size_t)t + 2];
        const float* p0 = pos + 3 * (size_t)i0;
        const float* p1 = pos + 3 * (size_t)i1;
        const float* p2 = pos + 3 * (size_t)i2;
        tris[3 * (size_t)p] = make_float4(p0[0], p0[1], p0[2], __uint_as_float(local));
        tris[3 * (size_t)p + 1] = make_float4(p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2], 0.0f);
        tris[3 * (size_t)p + 2] = make_float4(p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2], 0.0f);
    }
}

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t n = 0;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t count) {
        if (count <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) n = count;
        return e;
    }
};

int blocks_for(uint64_t n, int block = 256) { return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + block - 1) / block, 1u << 20)); }

}  // namespace

// Builds the reference BVH of every mesh (all non-empty; prims of mesh m at
// [prim_base[m], prim_base[m] + n_prims[m]) of the device bound arrays).
// Results stay on the device: breadth-first nodes, depth-first indices, final
// primitive order. Host vectors get per-mesh node counts.
struct DeviceBvh {
    DevBuf<float4> blo, bhi, cen;
    DevBuf<uint32_t> idx, idx2, flag, pre, front, back, block_sum, total, prim_mesh;
    DevBuf<int32_t> pos_task;
    DevBuf<Task> tasks, next;
    DevBuf<TaskAcc> acc;
    DevBuf<TaskState> st;
    DevBuf<BNode> nodes;
    DevBuf<uint32_t> size, isize, dfs, ifs, counters, mesh_prim_base;
    std::vector<uint32_t> level_first, level_count;
    std::vector<uint32_t> mesh_nodes, mesh_inodes;  // per mesh: nodes, interior nodes
    uint32_t n_prims = 0, n_meshes = 0, n_nodes = 0;
};

#define DTRY(expr)                                                            \
    do {                                                                      \
        cudaError_t _e = (expr);                                              \
        if (_e != cudaSuccess) return cuda_check(ctx, _e, #expr);             \
    } while (0)

static int build_device_bvh(pyre_ctx* ctx, DeviceBvh& B, const std::vector<uint32_t>& prim_base) {
    cudaStream_t st = ctx->stream;
    const uint32_t N = B.n_prims, M = B.n_meshes;
    DTRY(B.idx.alloc(N)); DTRY(B.idx2.alloc(N)); DTRY(B.flag.alloc(N)); DTRY(B.pre.alloc(N + 1));
    DTRY(B.front.alloc(N)); DTRY(B.back.alloc(N)); DTRY(B.prim_mesh.alloc(N)); DTRY(B.pos_task.alloc(N));
    const uint32_t scan_blocks = (N + 4 * kScanBlock - 1) / (4 * kScanBlock);
    DTRY(B.block_sum.alloc(std::max(scan_blocks, 1u))); DTRY(B.total.alloc(1));
    DTRY(B.nodes.alloc(2 * (size_t)N)); DTRY(B.counters.alloc(2)); DTRY(B.mesh_prim_base.alloc(M));
    DTRY(cudaMemcpyAsync(B.mesh_prim_base.p, prim_base.data(), M * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    k_prim_mesh<<<blocks_for(N), 256, 0, st>>>(B.mesh_prim_base.p, M, N, B.prim_mesh.p, B.pos_task.p, B.idx.p);
    // level 0: one task (and root node m) per mesh
    std::vector<Task> roots(M);
    for (uint32_t m = 0; m < M; ++m)
        roots[m] = Task{prim_base[m], m + 1 < M ? prim_base[m + 1] : N, m, m};
    DTRY(B.tasks.alloc(M));
    DTRY(cudaMemcpyAsync(B.tasks.p, roots.data(), M * sizeof(Task), cudaMemcpyHostToDevice, st));
    uint32_t n_tasks = M, node_count = M;
    B.level_first.clear(); B.level_count.clear();
    B.level_first.push_back(0); B.level_count.push_back(M);
    uint32_t* h_counters = nullptr;
    DTRY(cudaMallocHost(&h_counters, 2 * sizeof(uint32_t)));
    int rc = PYRE_OK;
    while (n_tasks > 0) {
        if ((rc = cuda_check(ctx, B.acc.alloc(n_tasks), "alloc"))) break;
        if ((rc = cuda_check(ctx, B.st.alloc(n_tasks), "alloc"))) break;
        if ((rc = cuda_check(ctx, B.next.alloc(2 * (size_t)n_tasks), "alloc"))) break;
        const int tb = blocks_for(n_tasks, 128);
        k_init_acc<<<tb, 128, 0, st>>>(B.acc.p, n_tasks);
        k_box<<<blocks_for(N), 256, 0, st>>>(B.pos_task.p, B.idx.p, B.blo.p, B.bhi.p, B.cen.p, N, B.acc.p);
        k_prepare<<<tb, 128, 0, st>>>(B.tasks.p, B.acc.p, n_tasks, B.st.p);
        k_bin<<<blocks_for(N), 256, 0, st>>>(B.pos_task.p, B.idx.p, B.blo.p, B.bhi.p, B.cen.p, N, B.st.p, B.acc.p);
        k_decide<<<tb, 128, 0, st>>>(B.tasks.p, B.acc.p, n_tasks, B.st.p);
        k_flags<<<blocks_for(N), 256, 0, st>>>(B.pos_task.p, B.idx.p, B.cen.p, N, B.st.p, B.flag.p);
        k_scan_local<<<std::max(scan_blocks, 1u), kScanBlock, 0, st>>>(B.flag.p, N, B.pre.p, B.block_sum.p);
        k_scan_sums<<<1, kScanBlock, 0, st>>>(B.block_sum.p, std::max(scan_blocks, 1u), B.total.p);
        k_scan_add<<<blocks_for(N + 1), 256, 0, st>>>(B.pre.p, N, B.block_sum.p, B.total.p);
        k_tables<<<blocks_for(N), 256, 0, st>>>(B.pos_task.p, B.tasks.p, B.st.p, B.flag.p, B.pre.p, N, B.front.p,
                                                B.back.p);
        k_scatter<<<blocks_for(N), 256, 0, st>>>(B.pos_task.p, B.tasks.p, B.st.p, B.flag.p, B.pre.p, B.front.p,
                                                 B.back.p, B.idx.p, N, B.idx2.p);
        std::swap(B.idx.p, B.idx2.p);
        std::swap(B.idx.n, B.idx2.n);
        h_counters[0] = 0;
        h_counters[1] = node_count;
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(B.counters.p, h_counters, 2 * sizeof(uint32_t),
                                                  cudaMemcpyHostToDevice, st), "counters"))) break;
        k_finish<<<tb, 128, 0, st>>>(B.tasks.p, B.acc.p, n_tasks, B.pre.p, B.st.p, B.nodes.p, B.next.p,
                                     B.counters.p);
        k_assign<<<blocks_for(N), 256, 0, st>>>(B.pos_task.p, B.st.p, N);
        if ((rc = cuda_check(ctx, cudaMemcpyAsync(h_counters, B.counters.p, 2 * sizeof(uint32_t),
                                                  cudaMemcpyDeviceToHost, st), "counters"))) break;
        if ((rc = cuda_check(ctx, cudaStreamSynchronize(st), "build level"))) break;
        n_tasks = h_counters[0];
        if (n_tasks) {
            B.level_first.push_back(node_count);
            B.level_count.push_back(n_tasks);
        }
        node_count = h_counters[1];
        std::swap(B.tasks.p, B.next.p);
        std::swap(B.tasks.n, B.next.n);
    }
    cudaFreeHost(h_counters);
    if (rc) return rc;
    B.n_nodes = node_count;
    // subtree sizes bottom-up, then depth-first indices top-down
    DTRY(B.size.alloc(node_count)); DTRY(B.isize.alloc(node_count));
    DTRY(B.dfs.alloc(node_count)); DTRY(B.ifs.alloc(node_count));
    for (size_t l = B.level_first.size(); l-- > 0;)
        k_sizes<<<blocks_for(B.level_count[l], 128), 128, 0, st>>>(B.nodes.p, B.level_first[l], B.level_count[l],
                                                                    B.size.p, B.isize.p);
    DTRY(cudaMemsetAsync(B.dfs.p, 0, M * sizeof(uint32_t), st));  // roots are nodes 0 .. M-1
    DTRY(cudaMemsetAsync(B.ifs.p, 0, M * sizeof(uint32_t), st));
    for (size_t l = 0; l < B.level_first.size(); ++l)
        k_order<<<blocks_for(B.level_count[l], 128), 128, 0, st>>>(B.nodes.p, B.level_first[l], B.level_count[l],
                                                                    B.size.p, B.isize.p, B.dfs.p, B.ifs.p);
    B.mesh_nodes.assign(M, 0);
    B.mesh_inodes.assign(M, 0);
    DTRY(cudaMemcpyAsync(B.mesh_nodes.data(), B.size.p, M * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    DTRY(cudaMemcpyAsync(B.mesh_inodes.data(), B.isize.p, M * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    DTRY(cudaStreamSynchronize(st));
    DTRY(cudaGetLastError());
    return PYRE_OK;
}

int device_build_blas(pyre_ctx* ctx, const pyre_scene_desc* desc, const std::vector<uint32_t>& mesh_ids,
                      DeviceBlas* out) {
    cudaStream_t st = ctx->stream;
    const uint32_t M = (uint32_t)mesh_ids.size();
    std::vector<uint32_t> prim_base(M);
    uint64_t n_tri = 0, n_vert = 0;
    for (uint32_t k = 0; k < M; ++k) {
        prim_base[k] = (uint32_t)n_tri;
        n_tri += desc->meshes[mesh_ids[k]].n_triangles;
        n_vert += desc->meshes[mesh_ids[k]].n_vertices;
    }
    if (n_tri >= (1ull << 31) || 3 * n_vert >= (1ull << 32))
        return set_error(ctx, PYRE_ERR_UNSUPPORTED, "scene too large for the device BVH build");
    // all meshes' vertices, and their indices rebased to the concatenation
    std::vector<uint32_t> vidx(3 * n_tri);
    std::vector<float> pos(3 * n_vert);
    uint64_t vb = 0, tb = 0;
    for (uint32_t k = 0; k < M; ++k) {
        const pyre_mesh_desc& md = desc->meshes[mesh_ids[k]];
        std::memcpy(pos.data() + 3 * vb, md.positions, 3 * (size_t)md.n_vertices * sizeof(float));
        for (uint64_t i = 0; i < 3ull * md.n_triangles; ++i) vidx[3 * tb + i] = (uint32_t)(vb + md.indices[i]);
        vb += md.n_vertices;
        tb += md.n_triangles;
    }
    DeviceBvh B;
    B.n_prims = (uint32_t)n_tri;
    B.n_meshes = M;
    DevBuf<float> d_pos;
    DevBuf<uint32_t> d_vidx;
    DTRY(d_pos.alloc(pos.size())); DTRY(d_vidx.alloc(vidx.size()));
    DTRY(cudaMemcpyAsync(d_pos.p, pos.data(), pos.size() * sizeof(float), cudaMemcpyHostToDevice, st));
    DTRY(cudaMemcpyAsync(d_vidx.p, vidx.data(), vidx.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    DTRY(B.blo.alloc(n_tri)); DTRY(B.bhi.alloc(n_tri)); DTRY(B.cen.alloc(n_tri));
    k_tri_bounds<<<blocks_for(n_tri), 256, 0, st>>>(d_pos.p, d_vidx.p, (uint32_t)n_tri, B.blo.p, B.bhi.p, B.cen.p);
    int rc = build_device_bvh(ctx, B, prim_base);
    if (rc) return rc;
    // node bases: interior nodes of each mesh (one node for a leaf root)
    std::vector<uint32_t> node_base(M);
    uint64_t total = 0;
    for (uint32_t k = 0; k < M; ++k) {
        node_base[k] = (uint32_t)total;
        total += std::max(B.mesh_inodes[k], 1u);
    }
    std::vector<BNode> roots(M);
    DTRY(cudaMemcpyAsync(roots.data(), B.nodes.p, M * sizeof(BNode), cudaMemcpyDeviceToHost, st));
    DevBuf<uint32_t> d_node_base;
    DTRY(d_node_base.alloc(M));
    DTRY(cudaMemcpyAsync(d_node_base.p, node_base.data(), M * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
    GpuNode* d_nodes = nullptr;
    float4* d_tris = nullptr;
    DTRY(cudaMalloc(&d_nodes, std::max<uint64_t>(total, 1) * sizeof(GpuNode)));
    cudaError_t e = cudaMalloc(&d_tris, 3 * n_tri * sizeof(float4));
    if (e != cudaSuccess) { cudaFree(d_nodes); return cuda_check(ctx, e, "cudaMalloc(triangles)"); }
    k_emit_gpu<<<blocks_for(B.n_nodes), 256, 0, st>>>(B.nodes.p, B.n_nodes, M, B.ifs.p, d_node_base.p, d_nodes);
    k_emit_tris<<<blocks_for(n_tri), 256, 0, st>>>(B.idx.p, (uint32_t)n_tri, B.prim_mesh.p, B.mesh_prim_base.p,
                                                    d_pos.p, d_vidx.p, d_tris);
    e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) { cudaFree(d_nodes); cudaFree(d_tris); return cuda_check(ctx, e, "device BVH emit"); }
    out->nodes = d_nodes;
    out->n_nodes = total;
    out->tris = d_tris;
    out->root.assign(M, 0);
    out->box.assign(M, Aabb{});
    for (uint32_t k = 0; k < M; ++k) {
        out->root[k] = (int32_t)node_base[k];
        out->box[k].lo = mk3(roots[k].lo[0], roots[k].lo[1], roots[k].lo[2]);
        out->box[k].hi = mk3(roots[k].hi[0], roots[k].hi[1], roots[k].hi[2]);
    }
    return PYRE_OK;
}

}  // namespace pyre

using namespace pyre;

extern "C" int pyre_bvh_build_device(pyre_ctx* ctx, const float* positions, uint32_t n_vertices,
                                     const uint32_t* indices, uint32_t n_triangles, pyre_bvh2_node* nodes_out,
                                     uint32_t* prim_indices_out, uint32_t* n_nodes_out) {
    NvtxRange nvtx("pyre_bvh_build_device");
    if (!ctx || !positions || !indices || !nodes_out || !prim_indices_out || !n_nodes_out)
        return set_error(ctx, PYRE_ERR_INVALID, "pyre_bvh_build_device: NULL argument");
    for (uint64_t i = 0; i < 3ull * n_triangles; ++i)
        if (indices[i] >= n_vertices) return set_error(ctx, PYRE_ERR_INVALID, "index out of range");
    *n_nodes_out = 0;
    if (n_triangles == 0) return PYRE_OK;
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    DeviceBvh B;
    B.n_prims = n_triangles;
    B.n_meshes = 1;
    DevBuf<float> d_pos;
    DevBuf<uint32_t> d_idx;
    DTRY(d_pos.alloc(3 * (size_t)n_vertices)); DTRY(d_idx.alloc(3 * (size_t)n_triangles));
    DTRY(cudaMemcpyAsync(d_pos.p, positions, 3 * (size_t)n_vertices * 4, cudaMemcpyHostToDevice, st));
    DTRY(cudaMemcpyAsync(d_idx.p, indices, 3 * (size_t)n_triangles * 4, cudaMemcpyHostToDevice, st));
    DTRY(B.blo.alloc(n_triangles)); DTRY(B.bhi.alloc(n_triangles)); DTRY(B.cen.alloc(n_triangles));
    k_tri_bounds<<<blocks_for(n_triangles), 256, 0, st>>>(d_pos.p, d_idx.p, n_triangles, B.blo.p, B.bhi.p, B.cen.p);
    std::vector<uint32_t> base{0};
    int rc = build_device_bvh(ctx, B, base);
    if (rc) return rc;
    DevBuf<pyre_bvh2_node> d_out;
    DevBuf<uint32_t> d_prim, d_node_base;
    DTRY(d_out.alloc(B.n_nodes)); DTRY(d_prim.alloc(n_triangles)); DTRY(d_node_base.alloc(1));
    DTRY(cudaMemsetAsync(d_node_base.p, 0, sizeof(uint32_t), st));
    k_emit_ref<<<blocks_for(B.n_nodes), 256, 0, st>>>(B.nodes.p, B.n_nodes, B.dfs.p, d_node_base.p,
                                                       B.mesh_prim_base.p, d_out.p);
    k_emit_prims<<<blocks_for(n_triangles), 256, 0, st>>>(B.idx.p, n_triangles, B.prim_mesh.p, B.mesh_prim_base.p,
                                                          d_prim.p);
    DTRY(cudaMemcpyAsync(nodes_out, d_out.p, B.n_nodes * sizeof(pyre_bvh2_node), cudaMemcpyDeviceToHost, st));
    DTRY(cudaMemcpyAsync(prim_indices_out, d_prim.p, n_triangles * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    DTRY(cudaStreamSynchronize(st));
    DTRY(cudaGetLastError());
    *n_nodes_out = B.n_nodes;
    return PYRE_OK;
}
