// Host BVH code under AddressSanitizer / UndefinedBehaviorSanitizer: builds
// the reference BVH of random and degenerate triangle sets, validates it,
// collapses it into binary and 4-/8-wide device nodes and checks that every
// triangle slot is reachable exactly once. Exit status 0 on success; the
// sanitizers abort on any memory or undefined-behaviour error.
#include <cstdio>
#include <random>
#include <vector>

#include "../../pyre_gb300/csrc/bvh_host.h"

using namespace pyre;

static int fail(const char* what, int n) {
    std::fprintf(stderr, "FAIL %s (n=%d)\n", what, n);
    return 1;
}

static int check(const std::vector<float>& pos, const std::vector<uint32_t>& idx) {
    const uint32_t nt = (uint32_t)(idx.size() / 3);
    std::vector<Aabb> b;
    std::vector<f3> c;
    triangle_bounds(pos.data(), idx.data(), nt, b, c);
    std::vector<pyre_bvh2_node> nodes;
    std::vector<uint32_t> prim;
    build_bvh2(b, c, nodes, prim);
    std::string why;
    if (!validate_bvh2(nodes.data(), (uint32_t)nodes.size(), prim.data(), nt, &why)) return fail(why.c_str(), (int)nt);
    // the C entry point gives the same array
    std::vector<pyre_bvh2_node> n2(2 * (size_t)nt);
    std::vector<uint32_t> p2(nt);
    uint32_t cnt = 0;
    if (pyre_bvh_build(pos.data(), (uint32_t)(pos.size() / 3), idx.data(), nt, n2.data(), p2.data(), &cnt) != 0 ||
        cnt != nodes.size() || p2 != prim)
        return fail("pyre_bvh_build differs", (int)nt);
    std::vector<GpuNode> bin;
    collapse_bvh2(nodes.data(), (uint32_t)nodes.size(), 0, 0, bin);
    for (int w : {4, 8}) {
        std::vector<float> wide;
        const int32_t root = collapse_wide(bin, 0, w, wide);
        const size_t stride = (size_t)PYRE_WIDE_FIELDS * w;
        if (root != 0 || wide.size() % stride) return fail("wide layout", (int)nt);
        std::vector<int> seen(nt, 0);
        std::vector<int32_t> stack{0};
        while (!stack.empty()) {
            const int32_t n = stack.back();
            stack.pop_back();
            if (n < 0 || (size_t)(n + 1) * stride > wide.size()) return fail("wide child out of range", (int)nt);
            const int32_t* I = reinterpret_cast<const int32_t*>(wide.data() + (size_t)n * stride);
            for (int k = 0; k < w; ++k) {
                const int32_t ch = I[6 * w + k], ct = I[7 * w + k];
                if (ch < 0) continue;
                if (ct == 0) { stack.push_back(ch); continue; }
                for (int32_t s = ch; s < ch + ct; ++s) {
                    if (s < 0 || (uint32_t)s >= nt) return fail("wide leaf out of range", (int)nt);
                    seen[(size_t)s] += 1;
                }
            }
        }
        // leaves of the reference BVH cover every slot once, except primitives
        // of a coincident-centroid leaf beyond the 65535 a leaf can hold
        for (uint32_t s = 0; s < nt; ++s)
            if (seen[s] > 1) return fail("slot reached twice", (int)nt);
    }
    return 0;
}

int main() {
    std::mt19937 rng(7);
    std::uniform_real_distribution<float> u(-1.0f, 1.0f);
    int bad = 0;
    for (int n : {1, 2, 3, 8, 9, 17, 100, 1000, 5000}) {
        std::vector<float> pos(9 * (size_t)n);
        std::vector<uint32_t> idx(3 * (size_t)n);
        for (size_t i = 0; i < pos.size(); ++i) pos[i] = u(rng);
        for (size_t i = 0; i < idx.size(); ++i) idx[i] = (uint32_t)i;
        bad += check(pos, idx);  // triangle soup
        std::vector<float> same(9 * (size_t)n, 0.25f);
        bad += check(same, idx);  // all centroids coincide
        std::vector<float> flat(pos);
        for (size_t i = 1; i < flat.size(); i += 3) flat[i] = 0.0f;  // one plane
        bad += check(flat, idx);
        std::vector<float> clus(pos);
        for (size_t i = 0; i < clus.size(); ++i) clus[i] = (float)((i / 9) % 3);  // three clusters
        bad += check(clus, idx);
    }
    std::printf(bad ? "failures: %d\n" : "ok\n", bad);
    return bad ? 1 : 0;
}
