// bvh_host.cpp — host BVH build (reference algorithm) and device collapse.
//
// The binned SAH build reproduces Bvh::build of the Pyre renderer
// (crates/pyre/src/geometry/bvh.rs:45-64,180-409) decision for decision —
// 12 bins on the longest centroid axis, cost 1 + 2(nL·AL + nR·AR)/A, leaves of
// at most 8 primitives, midpoint and equal-count fallbacks — so that a BVH
// built here and one handed over by the Rust host (Bvh::nodes()) are the same
// array. The recursion is replaced by an explicit task stack that emits nodes
// in the same depth-first pre-order.
#include "bvh_host.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <string>

namespace pyre {

namespace {

const int kBins = 12;
const float kInf = std::numeric_limits<float>::infinity();

inline Aabb empty_box() { Aabb b; b.lo = splat3(kInf); b.hi = splat3(-kInf); return b; }
inline Aabb unite(const Aabb& a, const Aabb& b) { Aabb r; r.lo = vmin3(a.lo, b.lo); r.hi = vmax3(a.hi, b.hi); return r; }
inline Aabb grow(const Aabb& a, f3 p) { Aabb r; r.lo = vmin3(a.lo, p); r.hi = vmax3(a.hi, p); return r; }
inline float area(const Aabb& b) {
    f3 d = b.hi - b.lo;
    return 2.0f * (d.x * d.y + d.x * d.z + d.y * d.z);
}
inline float comp(f3 v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
inline int widest(f3 v) {
    if (v.x >= v.y && v.x >= v.z) return 0;
    return v.y >= v.z ? 1 : 2;
}
// Rust `f32 as i32`: saturating, NaN -> 0.
inline int32_t sat_i32(float f) {
    if (std::isnan(f)) return 0;
    if (f >= 2147483647.0f) return 2147483647;
    if (f <= -2147483648.0f) return -2147483647 - 1;
    return (int32_t)f;
}

struct Task {
    uint32_t start, end;
    int64_t patch_parent;  // node whose `offset` becomes this subtree's index, or -1
};

}  // namespace

void triangle_bounds(const float* positions, const uint32_t* indices, uint32_t n_triangles,
                     std::vector<Aabb>& bounds, std::vector<f3>& centroids) {
    bounds.resize(n_triangles);
    centroids.resize(n_triangles);
    for (uint32_t t = 0; t < n_triangles; ++t) {
        const float* p0 = positions + 3 * (size_t)indices[3 * (size_t)t];
        const float* p1 = positions + 3 * (size_t)indices[3 * (size_t)t + 1];
        const float* p2 = positions + 3 * (size_t)indices[3 * (size_t)t + 2];
        f3 a = mk3(p0[0], p0[1], p0[2]), b = mk3(p1[0], p1[1], p1[2]), c = mk3(p2[0], p2[1], p2[2]);
        Aabb box; box.lo = a; box.hi = a;
        box = grow(grow(box, b), c);
        bounds[t] = box;
        centroids[t] = (a + b + c) / 3.0f;
    }
}

void build_bvh2(const std::vector<Aabb>& pb, const std::vector<f3>& pc,
                std::vector<pyre_bvh2_node>& nodes, std::vector<uint32_t>& idx, uint32_t max_leaf) {
    const uint32_t n_all = (uint32_t)pb.size();
    idx.resize(n_all);
    for (uint32_t i = 0; i < n_all; ++i) idx[i] = i;
    nodes.clear();
    nodes.reserve(2 * std::max<size_t>(n_all, 1));
    if (n_all == 0) return;

    auto emit = [&](const Aabb& box, uint32_t offset, uint16_t count, uint8_t axis) {
        pyre_bvh2_node nd;
        std::memset(&nd, 0, sizeof nd);
        nd.bounds_min[0] = box.lo.x; nd.bounds_min[1] = box.lo.y; nd.bounds_min[2] = box.lo.z;
        nd.bounds_max[0] = box.hi.x; nd.bounds_max[1] = box.hi.y; nd.bounds_max[2] = box.hi.z;
        nd.offset = offset;
        nd.n_primitives = count;
        nd.axis = axis;
        nodes.push_back(nd);
        return (uint32_t)nodes.size() - 1;
    };
    // Split point partition (bvh.rs:389-409): swap-from-the-end, not stable.
    auto partition = [&](uint32_t start, uint32_t end, int axis, float pos) {
        size_t l = start, r = end;
        while (l < r) {
            if (comp(pc[idx[l]], axis) < pos) ++l;
            else { --r; std::swap(idx[l], idx[r]); }
        }
        return (uint32_t)l;
    };

    std::vector<Task> stack;
    stack.push_back(Task{0, n_all, -1});
    while (!stack.empty()) {
        Task task = stack.back();
        stack.pop_back();
        if (task.patch_parent >= 0) nodes[(size_t)task.patch_parent].offset = (uint32_t)nodes.size();
        const uint32_t start = task.start, end = task.end, n = end - start;

        Aabb box = empty_box(), cbox = empty_box();
        for (uint32_t k = start; k < end; ++k) {
            box = unite(box, pb[idx[k]]);
            cbox = grow(cbox, pc[idx[k]]);
        }
        if (n == 1) { emit(box, start, 1, 0); continue; }
        const f3 cdiag = cbox.hi - cbox.lo;
        const int axis = widest(cdiag);
        const float extent = comp(cdiag, axis);
        if (extent < 1e-9f) { emit(box, start, (uint16_t)std::min<uint32_t>(n, 65535u), 0); continue; }

        uint32_t bin_n[kBins];
        Aabb bin_box[kBins];
        for (int i = 0; i < kBins; ++i) { bin_n[i] = 0; bin_box[i] = empty_box(); }
        const float cmin = comp(cbox.lo, axis);
        const float scale = (float)kBins / extent;
        for (uint32_t k = start; k < end; ++k) {
            int32_t b = sat_i32((comp(pc[idx[k]], axis) - cmin) * scale);
            b = std::min(std::max(b, 0), kBins - 1);
            bin_n[b] += 1;
            bin_box[b] = unite(bin_box[b], pb[idx[k]]);
        }
        // Prefix (left) and suffix (right) sweeps over the 11 bin boundaries.
        uint32_t ln[kBins - 1], rn[kBins - 1];
        Aabb lb[kBins - 1], rb[kBins - 1];
        {
            uint32_t c = 0; Aabb acc = empty_box();
            for (int i = 0; i < kBins - 1; ++i) { c += bin_n[i]; acc = unite(acc, bin_box[i]); ln[i] = c; lb[i] = acc; }
            c = 0; acc = empty_box();
            for (int i = kBins - 2; i >= 0; --i) { c += bin_n[i + 1]; acc = unite(acc, bin_box[i + 1]); rn[i] = c; rb[i] = acc; }
        }
        const float parent_area = std::fmax(area(box), 1e-9f);
        float best = kInf;
        int best_i = 0;
        for (int i = 0; i < kBins - 1; ++i) {
            if (ln[i] == 0 || rn[i] == 0) continue;
            float cost = 1.0f + 2.0f * ((float)ln[i] * area(lb[i]) + (float)rn[i] * area(rb[i])) / parent_area;
            if (cost < best) { best = cost; best_i = i; }
        }

        uint32_t mid;
        if (!std::isfinite(best)) {
            mid = partition(start, end, axis, cmin + 0.5f * extent);
            if (mid == start || mid == end) {
                if (n <= max_leaf) { emit(box, start, (uint16_t)n, 0); continue; }
                mid = start + n / 2;
            }
        } else {
            if (n <= max_leaf && best >= 2.0f * (float)n) { emit(box, start, (uint16_t)n, 0); continue; }
            mid = partition(start, end, axis, cmin + (float)(best_i + 1) * extent / (float)kBins);
            if (mid == start || mid == end) {
                if (n <= max_leaf) { emit(box, start, (uint16_t)n, 0); continue; }
                mid = start + n / 2;
            }
        }
        uint32_t self = emit(box, 0, 0, (uint8_t)axis);
        stack.push_back(Task{mid, end, (int64_t)self});  // right subtree, visited second
        stack.push_back(Task{start, mid, -1});           // left subtree = self + 1
    }
}

bool validate_bvh2(const pyre_bvh2_node* nodes, uint32_t n_nodes, const uint32_t* prim, uint32_t n_prims,
                   std::string* why) {
    if (n_prims == 0) return n_nodes == 0;
    if (n_nodes == 0 || nodes == nullptr || prim == nullptr) { *why = "BVH arrays missing"; return false; }
    std::vector<uint8_t> seen(n_prims, 0);
    std::vector<uint32_t> stack{0};
    uint64_t visited = 0;
    while (!stack.empty()) {
        uint32_t i = stack.back();
        stack.pop_back();
        if (i >= n_nodes) { *why = "BVH child index out of range"; return false; }
        if (++visited > n_nodes) { *why = "BVH has a cycle"; return false; }
        const pyre_bvh2_node& nd = nodes[i];
        if (nd.n_primitives > 0) {
            if ((uint64_t)nd.offset + nd.n_primitives > n_prims) { *why = "BVH leaf range out of range"; return false; }
            for (uint32_t k = nd.offset; k < nd.offset + nd.n_primitives; ++k) {
                if (prim[k] >= n_prims) { *why = "BVH primitive index out of range"; return false; }
                if (seen[k]++) { *why = "BVH leaf ranges overlap"; return false; }
            }
        } else {
            if (i + 1 >= n_nodes || nd.offset >= n_nodes || nd.offset <= i) { *why = "BVH interior node links invalid"; return false; }
            stack.push_back(nd.offset);
            stack.push_back(i + 1);
        }
    }
    for (uint32_t k = 0; k < n_prims; ++k)
        if (!seen[k]) { *why = "BVH does not reference every primitive"; return false; }
    return true;
}

namespace {
inline Aabb node_box(const pyre_bvh2_node& n) {
    Aabb b;
    b.lo = mk3(n.bounds_min[0], n.bounds_min[1], n.bounds_min[2]);
    b.hi = mk3(n.bounds_max[0], n.bounds_max[1], n.bounds_max[2]);
    return b;
}
inline void set_child(GpuNode& g, int slot, const Aabb& b, int32_t child, int32_t count) {
    float* xy = slot == 0 ? g.a : g.b;
    xy[0] = b.lo.x; xy[1] = b.hi.x; xy[2] = b.lo.y; xy[3] = b.hi.y;
    g.c[2 * slot] = b.lo.z; g.c[2 * slot + 1] = b.hi.z;
    g.d[slot] = child;
    g.d[2 + slot] = count;
}
}  // namespace

void set_gpu_child(GpuNode& g, int slot, const Aabb& box, int32_t child, int32_t count) {
    set_child(g, slot, box, child, count);
}

Aabb collapse_bvh2(const pyre_bvh2_node* nodes, uint32_t n_nodes, int32_t node_base, int32_t slot_base,
                   std::vector<GpuNode>& out) {
    Aabb root = node_box(nodes[0]);
    if (nodes[0].n_primitives > 0) {
        GpuNode g;
        std::memset(&g, 0, sizeof g);
        set_child(g, 0, root, slot_base + (int32_t)nodes[0].offset, nodes[0].n_primitives);
        Aabb none; none.lo = splat3(kInf); none.hi = splat3(-kInf);
        set_child(g, 1, none, -1, 0);
        out.push_back(g);
        return root;
    }
    // Interior reference nodes map to device nodes in DFS order.
    std::vector<int32_t> map(n_nodes, -1);
    int32_t next = node_base;
    for (uint32_t i = 0; i < n_nodes; ++i)
        if (nodes[i].n_primitives == 0) map[i] = next++;
    size_t first = out.size();
    out.resize(first + (size_t)(next - node_base));
    for (uint32_t i = 0; i < n_nodes; ++i) {
        if (nodes[i].n_primitives != 0) continue;
        GpuNode& g = out[first + (size_t)(map[i] - node_base)];
        std::memset(&g, 0, sizeof g);
        const uint32_t kids[2] = {i + 1, nodes[i].offset};
        for (int s = 0; s < 2; ++s) {
            const pyre_bvh2_node& c = nodes[kids[s]];
            if (c.n_primitives > 0) set_child(g, s, node_box(c), slot_base + (int32_t)c.offset, c.n_primitives);
            else set_child(g, s, node_box(c), map[kids[s]], 0);
        }
    }
    return root;
}

}  // namespace pyre

namespace pyre {
namespace {
struct WideChild {
    Aabb box;
    int32_t child, count;  // binary node index (count == 0) or leaf slot/count
};
inline float half_area(const Aabb& b) {
    const float dx = b.hi.x - b.lo.x, dy = b.hi.y - b.lo.y, dz = b.hi.z - b.lo.z;
    return dx * dy + dy * dz + dz * dx;
}
inline void binary_children(const GpuNode& g, std::vector<WideChild>& kids) {
    for (int s = 0; s < 2; ++s) {
        if (g.d[s] < 0) continue;
        const float* xy = s == 0 ? g.a : g.b;
        WideChild c;
        c.box.lo = mk3(xy[0], xy[2], g.c[2 * s]);
        c.box.hi = mk3(xy[1], xy[3], g.c[2 * s + 1]);
        c.child = g.d[s];
        c.count = g.d[2 + s];
        kids.push_back(c);
    }
}
}  // namespace

int32_t collapse_wide(const std::vector<GpuNode>& bin, int32_t root, int width, std::vector<float>& out) {
    const size_t stride = (size_t)PYRE_WIDE_FIELDS * width;
    // explicit DFS: (binary node, wide slot reserved for it)
    std::vector<std::pair<int32_t, int32_t>> todo;
    auto reserve = [&]() {
        const int32_t w = (int32_t)(out.size() / stride);
        out.resize(out.size() + stride, 0.0f);
        return w;
    };
    const int32_t wroot = reserve();
    todo.push_back({root, wroot});
    std::vector<WideChild> kids;
    while (!todo.empty()) {
        const auto [b, w] = todo.back();
        todo.pop_back();
        kids.clear();
        binary_children(bin[(size_t)b], kids);
        while ((int)kids.size() < width) {
            int best = -1;
            float area = -1.0f;
            for (int k = 0; k < (int)kids.size(); ++k)
                if (kids[k].count == 0 && half_area(kids[k].box) > area) { area = half_area(kids[k].box); best = k; }
            if (best < 0) break;
            const int32_t open = kids[best].child;
            kids.erase(kids.begin() + best);
            std::vector<WideChild> grand;
            binary_children(bin[(size_t)open], grand);
            kids.insert(kids.begin() + best, grand.begin(), grand.end());
        }
        // reserve the interior children first (pre-order: children follow the parent),
        // pushing them so the first child is expanded next
        std::vector<int32_t> wide_of(kids.size(), -1);
        for (size_t k = 0; k < kids.size(); ++k)
            if (kids[k].count == 0) wide_of[k] = reserve();
        for (size_t k = kids.size(); k-- > 0;)
            if (kids[k].count == 0) todo.push_back({kids[k].child, wide_of[k]});
        float* N = out.data() + (size_t)w * stride;
        int32_t* I = reinterpret_cast<int32_t*>(N);
        for (int k = 0; k < width; ++k) {
            const bool used = k < (int)kids.size();
            const Aabb bx = used ? kids[k].box : Aabb{splat3(kInf), splat3(-kInf)};
            N[0 * width + k] = bx.lo.x; N[1 * width + k] = bx.hi.x;
            N[2 * width + k] = bx.lo.y; N[3 * width + k] = bx.hi.y;
            N[4 * width + k] = bx.lo.z; N[5 * width + k] = bx.hi.z;
            I[6 * width + k] = !used ? -1 : (kids[k].count == 0 ? wide_of[k] : kids[k].child);
            I[7 * width + k] = used ? kids[k].count : 0;
        }
    }
    return wroot;
}

}  // namespace pyre

extern "C" int pyre_bvh_build(const float* positions, uint32_t n_vertices, const uint32_t* indices,
                              uint32_t n_triangles, pyre_bvh2_node* nodes_out, uint32_t* prim_indices_out,
                              uint32_t* n_nodes_out) {
    using namespace pyre;
    if (!positions || !indices || !nodes_out || !prim_indices_out || !n_nodes_out) return PYRE_ERR_INVALID;
    for (uint64_t i = 0; i < 3ull * n_triangles; ++i)
        if (indices[i] >= n_vertices) return PYRE_ERR_INVALID;
    std::vector<Aabb> bounds;
    std::vector<f3> cents;
    triangle_bounds(positions, indices, n_triangles, bounds, cents);
    std::vector<pyre_bvh2_node> nodes;
    std::vector<uint32_t> prim;
    build_bvh2(bounds, cents, nodes, prim);
    std::memcpy(nodes_out, nodes.data(), nodes.size() * sizeof(pyre_bvh2_node));
    std::memcpy(prim_indices_out, prim.data(), prim.size() * sizeof(uint32_t));
    *n_nodes_out = (uint32_t)nodes.size();
    return PYRE_OK;
}
