// CPU mesh preprocessing of the scene driver: watertightness test
// (src/scene.cpp:170-198) and the LBVH build/refit whose node layout the
// contact kernel traverses (src/mesh_lbvh.h:49-223, src/mesh_bvh.h:142-181).
#include <algorithm>
#include <cstring>
#include <utility>

#include "solver.h"

namespace xpbd {

bool tris_watertight(const uint32_t* tris, size_t num_tris, size_t num_verts) {
    if (num_tris == 0 || num_verts == 0) return false;
    std::vector<std::pair<uint32_t, uint32_t>> edges;
    edges.reserve(num_tris * 3);
    for (size_t t = 0; t < num_tris; t++)
        for (int k = 0; k < 3; k++) {
            uint32_t a = tris[t * 3 + k], b = tris[t * 3 + (k + 1) % 3];
            edges.emplace_back(std::min(a, b), std::max(a, b));
        }
    std::sort(edges.begin(), edges.end());
    for (size_t i = 0; i < edges.size();) {
        size_t j = i + 1;
        while (j < edges.size() && edges[j] == edges[i]) j++;
        if (j - i != 2) return false;  // every edge shared by exactly two triangles
        i = j;
    }
    return true;
}

static inline uint32_t spread10(uint32_t v) {  // interleave 10 bits with two zero bits
    v &= 0x3ffu;
    v = (v ^ (v << 16)) & 0xff0000ffu;
    v = (v ^ (v << 8)) & 0x0300f00fu;
    v = (v ^ (v << 4)) & 0x030c30c3u;
    v = (v ^ (v << 2)) & 0x09249249u;
    return v;
}
static inline uint32_t quantize1024(float f) {
    int i = (int)(f * 1024.0f);
    return (uint32_t)std::max(0, std::min(1023, i));
}
static inline uint32_t as_u32(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
static inline float as_f32(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

void HostBvh::build(const float* pts, const uint32_t* tris, size_t num_tris) {
    const uint32_t n = (uint32_t)num_tris;
    std::vector<float> lo(n * 3), hi(n * 3);
    float tlo[3] = {1e30f, 1e30f, 1e30f}, thi[3] = {-1e30f, -1e30f, -1e30f};
    for (uint32_t t = 0; t < n; t++) {
        for (int a = 0; a < 3; a++) lo[t * 3 + a] = hi[t * 3 + a] = pts[tris[t * 3] * 3 + a];
        for (int k = 1; k < 3; k++)
            for (int a = 0; a < 3; a++) {
                float c = pts[tris[t * 3 + k] * 3 + a];
                lo[t * 3 + a] = std::min(lo[t * 3 + a], c);
                hi[t * 3 + a] = std::max(hi[t * 3 + a], c);
            }
        for (int a = 0; a < 3; a++) {
            tlo[a] = std::min(tlo[a], lo[t * 3 + a]);
            thi[a] = std::max(thi[a], hi[t * 3 + a]);
        }
    }
    float inv[3];
    for (int a = 0; a < 3; a++) inv[a] = 1.0f / ((thi[a] - tlo[a]) + 0.0001f);
    std::vector<std::pair<uint32_t, uint32_t>> items(n);  // (morton, triangle)
    for (uint32_t t = 0; t < n; t++) {
        uint32_t q[3];
        for (int a = 0; a < 3; a++) q[a] = quantize1024((0.5f * (lo[t * 3 + a] + hi[t * 3 + a]) - tlo[a]) * inv[a]);
        items[t] = {(spread10(q[2]) << 2) | (spread10(q[1]) << 1) | spread10(q[0]), t};
    }
    std::stable_sort(items.begin(), items.end(),
                     [](const std::pair<uint32_t, uint32_t>& a, const std::pair<uint32_t, uint32_t>& b) {
                         return a.first < b.first;
                     });
    prims.resize(n);
    for (uint32_t i = 0; i < n; i++) prims[i] = items[i].second;
    auto common = [&](uint32_t i) {  // leading common bits of keys i, i+1 as 64-bit values
        uint64_t x = (uint64_t)items[i].first ^ (uint64_t)items[i + 1].first;
        return x == 0 ? 64 : __builtin_clzll(x);
    };
    const uint32_t m = 2 * n;
    lowers.assign((size_t)m * 4, 0.0f);
    uppers.assign((size_t)m * 4, 0.0f);
    std::vector<uint32_t> lw(m, 0), uw(m, 0);
    std::vector<int> parent(m, -1), children(m, 0), rl(m, 0), rr(m, 0);
    for (uint32_t i = 0; i < n; i++) {
        for (int a = 0; a < 3; a++) {
            lowers[i * 4 + a] = lo[prims[i] * 3 + a];
            uppers[i * 4 + a] = hi[prims[i] * 3 + a];
        }
        lw[i] = i | (1u << 30);
        uw[i] = i + 1;
        rl[i] = rr[i] = (int)i;
    }
    // bottom-up: each node picks the side whose boundary has the longer common
    // prefix (ties by primitive parity); the second child to arrive merges bounds
    for (uint32_t i = 0; i < n; i++) {
        int node = (int)i;
        for (;;) {
            const int L = rl[node], R = rr[node];
            if (L == 0 && R == (int)n - 1) {
                root = (uint32_t)node;
                parent[node] = -1;
                break;
            }
            bool go_right;
            if (L == 0) {
                go_right = true;
            } else if (R != (int)n - 1 && common(R) >= common(L - 1)) {
                go_right = common(R) == common(L - 1) ? (((prims[L - 1] & 1u) ^ (prims[R] & 1u)) != 0) : true;
            } else {
                go_right = false;
            }
            int p;
            if (go_right) {
                p = R + (int)n;
                lw[p] = (uint32_t)node;
                rl[p] = L;
            } else {
                p = L + (int)n - 1;
                uw[p] = (uint32_t)node;
                rr[p] = R;
            }
            parent[node] = p;
            if (++children[p] == 1) break;
            const uint32_t a = lw[p] & 0x3FFFFFFFu, b = uw[p] & 0x3FFFFFFFu;
            for (int k = 0; k < 3; k++) {
                lowers[p * 4 + k] = std::min(lowers[a * 4 + k], lowers[b * 4 + k]);
                uppers[p * 4 + k] = std::max(uppers[a * 4 + k], uppers[b * 4 + k]);
            }
            node = p;
        }
    }
    // collapse small subtrees (<= 4 primitives) and deep nodes (>= 32) into leaves
    for (uint32_t ni = 0; ni < m; ni++) {
        if (children[ni] == 0 && ni >= n) continue;
        int depth = 1;
        for (int p = parent[ni]; p != -1; p = parent[p]) depth++;
        const int L = rl[ni], Rx = rr[ni] + 1;
        if (Rx - L <= 4 || depth >= 32) {
            lw[ni] = (uint32_t)L | (1u << 30);
            uw[ni] = (uint32_t)Rx;
        }
    }
    for (uint32_t ni = 0; ni < m; ni++) {
        lowers[ni * 4 + 3] = as_f32(lw[ni]);
        uppers[ni * 4 + 3] = as_f32(uw[ni]);
    }
}

void HostBvh::refit(const float* pts, const uint32_t* tris) {
    // post-order over the reachable tree with an explicit stack
    std::vector<std::pair<uint32_t, bool>> st;
    st.emplace_back(root, false);
    while (!st.empty()) {
        auto [ni, expanded] = st.back();
        st.pop_back();
        const uint32_t lw = as_u32(lowers[ni * 4 + 3]), uw = as_u32(uppers[ni * 4 + 3]);
        if ((lw >> 30) & 3u) {
            float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
            for (uint32_t pi = lw & 0x3FFFFFFFu; pi < (uw & 0x3FFFFFFFu); pi++)
                for (int k = 0; k < 3; k++)
                    for (int a = 0; a < 3; a++) {
                        float c = pts[tris[prims[pi] * 3 + k] * 3 + a];
                        lo[a] = std::min(lo[a], c);
                        hi[a] = std::max(hi[a], c);
                    }
            for (int a = 0; a < 3; a++) {
                lowers[ni * 4 + a] = lo[a];
                uppers[ni * 4 + a] = hi[a];
            }
        } else if (!expanded) {
            st.emplace_back(ni, true);
            st.emplace_back(uw, false);
            st.emplace_back(lw & 0x3FFFFFFFu, false);
        } else {
            const uint32_t a = lw & 0x3FFFFFFFu, b = uw;
            for (int k = 0; k < 3; k++) {
                lowers[ni * 4 + k] = std::min(lowers[a * 4 + k], lowers[b * 4 + k]);
                uppers[ni * 4 + k] = std::max(uppers[a * 4 + k], uppers[b * 4 + k]);
            }
        }
    }
}

}  // namespace xpbd
