// extern "C" shim around the reference's own CPU BVH code, compiled in place
// from the reference checkout (see oracle/Makefile, target `ref`). Test
// infrastructure only: pins oracle/xpbd_oracle.c's LBVH restatement and the
// product's GPU LBVH against vkx::MeshBvh::build / refit (src/mesh_bvh.h:40-69,
// 142-181) and MeshLbvhBuilder::build (src/mesh_lbvh.h:49-223).
#include <cstdint>
#include <cstring>
#include <vector>
#include "mesh_bvh.h"

extern "C" {

// lowers/uppers: 4 floats per node (xyz + packed uint32 bits in w), 2*num_tris nodes.
int ref_bvh_build(const float* pts, int64_t num_pts, const uint32_t* tris, int64_t num_tris,
                  float* lowers, float* uppers, uint32_t* prims, uint32_t* root) {
    std::vector<float> p(pts, pts + num_pts * 3);
    std::vector<uint32_t> t(tris, tris + num_tris * 3);
    vkx::MeshBvh bvh;
    bvh.build(p, t);
    for (size_t i = 0; i < bvh.lowers.size(); i++) {
        std::memcpy(lowers + i * 4, &bvh.lowers[i], 16);
        std::memcpy(uppers + i * 4, &bvh.uppers[i], 16);
    }
    for (size_t i = 0; i < bvh.primitive_indices.size(); i++) prims[i] = bvh.primitive_indices[i];
    *root = bvh.root;
    return int(bvh.lowers.size());
}

// Build, move the vertices to pts_new, refit; returns the refit node halves.
int ref_bvh_build_refit(const float* pts, const float* pts_new, int64_t num_pts, const uint32_t* tris,
                        int64_t num_tris, float* lowers, float* uppers) {
    std::vector<float> p(pts, pts + num_pts * 3);
    std::vector<uint32_t> t(tris, tris + num_tris * 3);
    vkx::MeshBvh bvh;
    bvh.build(p, t);
    for (int64_t i = 0; i < num_pts * 3; i++) bvh.points[i] = pts_new[i];
    bvh.refit();
    for (size_t i = 0; i < bvh.lowers.size(); i++) {
        std::memcpy(lowers + i * 4, &bvh.lowers[i], 16);
        std::memcpy(uppers + i * 4, &bvh.uppers[i], 16);
    }
    return int(bvh.lowers.size());
}

// Brute-force closest point over all triangles (mesh_bvh.h:296-321).
int ref_query_closest(const float* pts, int64_t num_pts, const uint32_t* tris, int64_t num_tris,
                      const float* p, float max_dist, uint32_t* face, float* point) {
    vkx::MeshBvh bvh;
    bvh.points.assign(pts, pts + num_pts * 3);
    bvh.indices.assign(tris, tris + num_tris * 3);
    return bvh.query_closest(p, max_dist, *face, point) ? 1 : 0;
}

}  // extern "C"
