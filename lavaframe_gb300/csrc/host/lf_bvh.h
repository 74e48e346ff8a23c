// Host BVH construction and flattening for the LavaFrame scene layout.
//
// The flat node array that reaches the device has to be byte-identical to what the
// reference host code produces (RadeonRays SplitBvh for meshes, RadeonRays Bvh for the
// instance level, BvhTranslator for the flatten), so the build keeps the same algorithm:
//  - bottom level (per mesh): binned object SAH, 64 bins, traversal cost 2.0, leaves below
//    4 primitives, no spatial splits (the reference's max_split_depth is 0, so its spatial
//    split search never runs: thirdparty/RadeonRays/split_bvh.cpp:75, Mesh.h:18);
//    two-pointer partition whose direction flips on (start+count)&1
//    (split_bvh.cpp:112-150); median fallback (split_bvh.cpp:158-173); right child built
//    before the left one, which fixes the packed primitive order (split_bvh.cpp:183-188).
//  - top level (instances): split at the midpoint of the centroid bounds on the widest
//    axis, one instance per leaf, left child first (bvh.cpp:68-243).
//  - flatten: depth-first, left child first, all bottom-level trees first, the top level
//    starting at topLevelIndex with 2*instances slots reserved (bvh_translator.cpp:35-117).
// Float min/max and the order in which boxes grow follow the reference exactly, because
// signed zeros make min/max order-dependent.
//
// What differs from the reference is engineering, not results: the trees are built into
// flat vectors (no node pointers or chunk archives), recursion is replaced by explicit
// stacks, and independent meshes are built in parallel.
#pragma once

#include <cfloat>
#include <vector>
#include "lf_types.h"

namespace lfbvh
{
    using LavaFrame::Vec3;

    struct bbox
    {
        bbox() : pmin(FLT_MAX, FLT_MAX, FLT_MAX), pmax(-FLT_MAX, -FLT_MAX, -FLT_MAX) {}
        explicit bbox(const Vec3& p) : pmin(p), pmax(p) {}

        Vec3 center() const { return (pmax + pmin) * 0.5f; }
        Vec3 extents() const { return pmax - pmin; }
        float surface_area() const
        {
            Vec3 e = extents();
            return 2.f * (e.x * e.y + e.x * e.z + e.y * e.z);
        }
        int maxdim() const
        {
            Vec3 e = extents();
            if (e.x >= e.y && e.x >= e.z) return 0;
            if (e.y >= e.x && e.y >= e.z) return 1;
            if (e.z >= e.x && e.z >= e.y) return 2;
            return 0;
        }
        void grow(const Vec3& p) { pmin = Vec3::Min(pmin, p); pmax = Vec3::Max(pmax, p); }
        void grow(const bbox& b) { pmin = Vec3::Min(pmin, b.pmin); pmax = Vec3::Max(pmax, b.pmax); }

        Vec3 pmin;
        Vec3 pmax;
    };

    // One node of a built (not yet flattened) tree. Internal: a/b are child node ids in
    // `BuiltBvh::nodes`. Leaf: a = first position in `packed`, b = primitive count.
    struct BuiltNode
    {
        bbox bounds;
        int leaf;
        int a, b;
    };

    struct BuiltBvh
    {
        std::vector<BuiltNode> nodes;   // allocation order; nodes[0] is the root
        std::vector<int> packed;        // primitive ids in leaf order
        bbox bounds;                    // union of all primitive boxes
        int NodeCount() const { return (int)nodes.size(); }
    };

    // Mesh level: binned SAH (64 bins, cost 2.0, leaf < 4 primitives).
    void BuildMeshBvh(const bbox* prim_bounds, int n, BuiltBvh& out);
    // Instance level: centroid-midpoint split, one primitive per leaf.
    void BuildInstanceBvh(const bbox* prim_bounds, int n, BuiltBvh& out);

    // 36-byte flat node, identical in layout and meaning to the reference's
    // BvhTranslator::Node (thirdparty/RadeonRays/bvh_translator.h:48-53):
    //  inner node:          LRLeaf = (left index, right index, 0)
    //  mesh-level leaf:     LRLeaf = (first packed triangle, triangle count, 1)
    //  instance-level leaf: LRLeaf = (mesh root node index, material id, -instance-1)
    // Indices are stored as floats, exact below 2^24.
    struct FlatNode
    {
        Vec3 bboxmin;
        Vec3 bboxmax;
        Vec3 LRLeaf;
    };
    static_assert(sizeof(FlatNode) == 36, "flat node layout");

    // Writes the tree of one mesh at nodes[root_index ...], returns the next free index.
    // Leaves refer to packed triangles offset by tri_offset.
    int FlattenMesh(const BuiltBvh& bvh, int root_index, int tri_offset, FlatNode* nodes);

    // Writes the instance tree at nodes[top_index ...]. instance_mesh_root[i] is the flat
    // index of the root of instance i's mesh, instance_material[i] its material id.
    void FlattenInstances(const BuiltBvh& tlas, int top_index, const int* instance_mesh_root,
                          const int* instance_material, FlatNode* nodes);
}
