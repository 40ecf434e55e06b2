// Host mesh preprocessing of the scene driver: the watertightness test of
// add_mesh (src/scene.cpp:170-198). The BVH is built and refit on the GPU
// (k_bvh.cu).
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

}  // namespace xpbd
