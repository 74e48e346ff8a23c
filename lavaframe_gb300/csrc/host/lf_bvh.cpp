// Host BVH build + flatten. Algorithm notes live in lf_bvh.h.
#include "lf_bvh.h"

#include <cmath>
#include <utility>

namespace lfbvh
{
namespace
{
    constexpr int kBins = 64;
    constexpr float kMeshTraversalCost = 2.0f;

    struct PrimRef
    {
        bbox bounds;
        Vec3 center;
        int idx;
    };

    struct Request
    {
        int start;
        int num;
        bbox bounds;
        bbox cbounds;
        int parent;   // built node id of the parent, -1 for the root
        int side;     // 0: left child of parent, 1: right child
    };

    struct ObjectSplit
    {
        int dim;
        float split;
        bool valid;
    };

    // Binned object SAH over the primitive range of `req`
    // (thirdparty/RadeonRays/split_bvh.cpp:196-313).
    ObjectSplit FindObjectSahSplit(const Request& req, const PrimRef* refs)
    {
        ObjectSplit res{0, 0.f, false};
        const Vec3 ce = req.cbounds.extents();
        if (Vec3::Dot(ce, ce) == 0.f)
            return res;

        bbox bin_box[kBins];
        int bin_cnt[kBins];
        bbox right_acc[kBins - 1];

        const float invarea = 1.f / req.bounds.surface_area();
        const Vec3 rootmin = req.cbounds.pmin;
        float best = FLT_MAX;
        int best_bin = -1;

        for (int axis = 0; axis < 3; ++axis)
        {
            const float lo = rootmin[axis];
            const float rng = ce[axis];
            const float inv_rng = 1.f / rng;
            if (rng == 0.f)
                continue;

            for (int i = 0; i < kBins; ++i)
            {
                bin_box[i] = bbox();
                bin_cnt[i] = 0;
            }
            for (int i = req.start; i < req.start + req.num; ++i)
            {
                float v = static_cast<float>(kBins) * ((refs[i].center[axis] - lo) * inv_rng);
                const float cap = static_cast<float>(kBins - 1);
                int b = (int)((cap < v) ? cap : v);
                ++bin_cnt[b];
                bin_box[b].grow(refs[i].bounds);
            }

            bbox acc;
            for (int i = kBins - 1; i > 0; --i)
            {
                acc.grow(bin_box[i]);
                right_acc[i - 1] = acc;
            }

            bbox left;
            int nl = 0, nr = req.num;
            for (int i = 0; i < kBins - 1; ++i)
            {
                left.grow(bin_box[i]);
                nl += bin_cnt[i];
                nr -= bin_cnt[i];
                float cost = kMeshTraversalCost +
                             (nl * left.surface_area() + nr * right_acc[i].surface_area()) * invarea;
                if (cost < best)
                {
                    res.dim = axis;
                    best_bin = i;
                    best = cost;
                }
            }
        }

        if (best_bin != -1)
        {
            res.split = rootmin[res.dim] + (best_bin + 1) * (ce[res.dim] / kBins);
            res.valid = true;
        }
        return res;
    }

    // Accessors that let one partition routine serve both levels: the mesh level
    // permutes PrimRef records, the instance level permutes an index array.
    struct MeshItems
    {
        PrimRef* refs;
        const Vec3& center(int i) const { return refs[i].center; }
        const bbox& box(int i) const { return refs[i].bounds; }
        void swap(int i, int j) const { std::swap(refs[i], refs[j]); }
    };
    struct InstanceItems
    {
        int* idx;
        const Vec3* centers;
        const bbox* boxes;
        const Vec3& center(int i) const { return centers[idx[i]]; }
        const bbox& box(int i) const { return boxes[idx[i]]; }
        void swap(int i, int j) const { std::swap(idx[i], idx[j]); }
    };

    // Two-pointer partition around `border` on `axis`; the side that is scanned first
    // alternates with the parity of start+count (split_bvh.cpp:112-150, bvh.cpp:326-398).
    // Returns the split position and leaves the four boxes grown in reference order.
    template <class Items>
    int Partition(const Items& it, const Request& req, int axis, float border,
                  bbox& lb, bbox& rb, bbox& lcb, bbox& rcb)
    {
        int splitidx = req.start;
        const bool near2far = ((req.num + req.start) & 0x1) != 0;
        auto first_side = [&](float c) { return near2far ? (c < border) : (c >= border); };
        auto second_side = [&](float c) { return near2far ? (c >= border) : (c < border); };

        if (req.cbounds.extents()[axis] > 0.f)
        {
            int first = req.start;
            int last = req.start + req.num;
            while (true)
            {
                while (first != last && first_side(it.center(first)[axis]))
                {
                    lb.grow(it.box(first));
                    lcb.grow(it.center(first));
                    ++first;
                }
                if (first == last--)
                    break;
                rb.grow(it.box(first));
                rcb.grow(it.center(first));
                while (first != last && second_side(it.center(last)[axis]))
                {
                    rb.grow(it.box(last));
                    rcb.grow(it.center(last));
                    --last;
                }
                if (first == last)
                    break;
                lb.grow(it.box(last));
                lcb.grow(it.center(last));
                it.swap(first++, last);
            }
            splitidx = first;
        }

        if (splitidx == req.start || splitidx == req.start + req.num)
        {
            // Median fallback; boxes keep whatever the scan above already added.
            splitidx = req.start + (req.num >> 1);
            for (int i = req.start; i < splitidx; ++i)
            {
                lb.grow(it.box(i));
                lcb.grow(it.center(i));
            }
            for (int i = splitidx; i < req.start + req.num; ++i)
            {
                rb.grow(it.box(i));
                rcb.grow(it.center(i));
            }
        }
        return splitidx;
    }

    int AllocNode(BuiltBvh& out, const Request& req)
    {
        int id = (int)out.nodes.size();
        out.nodes.push_back(BuiltNode{req.bounds, 0, -1, -1});
        if (req.parent >= 0)
        {
            if (req.side == 0) out.nodes[req.parent].a = id;
            else out.nodes[req.parent].b = id;
        }
        return id;
    }
}

void BuildMeshBvh(const bbox* prim_bounds, int n, BuiltBvh& out)
{
    out.nodes.clear();
    out.packed.clear();
    out.bounds = bbox();
    for (int i = 0; i < n; ++i)
        out.bounds.grow(prim_bounds[i]);

    std::vector<PrimRef> refs(n);
    bbox cb;
    for (int i = 0; i < n; ++i)
    {
        refs[i] = PrimRef{prim_bounds[i], prim_bounds[i].center(), i};
        cb.grow(prim_bounds[i].center());
    }
    out.nodes.reserve(n > 0 ? 2 * n : 1);
    out.packed.reserve(n);

    MeshItems items{refs.data()};
    std::vector<Request> stack;
    stack.push_back(Request{0, n, out.bounds, cb, -1, 0});
    while (!stack.empty())
    {
        Request req = stack.back();
        stack.pop_back();
        int id = AllocNode(out, req);

        if (req.num < 4)
        {
            out.nodes[id].leaf = 1;
            out.nodes[id].a = (int)out.packed.size();
            out.nodes[id].b = req.num;
            for (int i = req.start; i < req.start + req.num; ++i)
                out.packed.push_back(refs[i].idx);
            continue;
        }

        int axis = req.cbounds.maxdim();
        float border = req.cbounds.center()[axis];
        ObjectSplit os = FindObjectSahSplit(req, refs.data());
        if (os.valid)
        {
            border = os.split;
            axis = os.dim;
        }

        bbox lb, rb, lcb, rcb;
        int split = Partition(items, req, axis, border, lb, rb, lcb, rcb);
        Request left{req.start, split - req.start, lb, lcb, id, 0};
        Request right{split, req.num - (split - req.start), rb, rcb, id, 1};
        // Right subtree first (LIFO: push left, then right).
        stack.push_back(left);
        stack.push_back(right);
    }
}

void BuildInstanceBvh(const bbox* prim_bounds, int n, BuiltBvh& out)
{
    out.nodes.clear();
    out.packed.clear();
    out.bounds = bbox();
    for (int i = 0; i < n; ++i)
        out.bounds.grow(prim_bounds[i]);

    std::vector<Vec3> centers(n);
    std::vector<int> idx(n);
    bbox cb;
    for (int i = 0; i < n; ++i)
    {
        Vec3 c = prim_bounds[i].center();
        cb.grow(c);
        centers[i] = c;
        idx[i] = i;
    }
    out.nodes.reserve(n > 0 ? 2 * n : 1);
    out.packed.reserve(n);

    InstanceItems items{idx.data(), centers.data(), prim_bounds};
    std::vector<Request> stack;
    stack.push_back(Request{0, n, out.bounds, cb, -1, 0});
    while (!stack.empty())
    {
        Request req = stack.back();
        stack.pop_back();
        int id = AllocNode(out, req);

        if (req.num < 2)
        {
            out.nodes[id].leaf = 1;
            out.nodes[id].a = (int)out.packed.size();
            out.nodes[id].b = req.num;
            for (int i = 0; i < req.num; ++i)
                out.packed.push_back(idx[req.start + i]);
            continue;
        }

        int axis = req.cbounds.maxdim();
        float border = req.cbounds.center()[axis];
        bbox lb, rb, lcb, rcb;
        int split = Partition(items, req, axis, border, lb, rb, lcb, rcb);
        Request left{req.start, split - req.start, lb, lcb, id, 0};
        Request right{split, req.num - (split - req.start), rb, rcb, id, 1};
        // Left subtree first (LIFO: push right, then left).
        stack.push_back(right);
        stack.push_back(left);
    }
}

namespace
{
    struct FlattenItem
    {
        int node;        // built node id
        int parent;      // flat index of the parent, -1 for the root
        int side;
    };

    template <class LeafFn>
    int FlattenPreorder(const BuiltBvh& bvh, int root_index, FlatNode* nodes, LeafFn leaf_fn)
    {
        int next = root_index;
        std::vector<FlattenItem> stack;
        stack.push_back(FlattenItem{0, -1, 0});
        while (!stack.empty())
        {
            FlattenItem it = stack.back();
            stack.pop_back();
            const BuiltNode& bn = bvh.nodes[it.node];
            int index = next++;
            FlatNode& fn = nodes[index];
            fn.bboxmin = bn.bounds.pmin;
            fn.bboxmax = bn.bounds.pmax;
            fn.LRLeaf = Vec3(0.f, 0.f, 0.f);
            if (it.parent >= 0)
            {
                if (it.side == 0) nodes[it.parent].LRLeaf.x = (float)index;
                else nodes[it.parent].LRLeaf.y = (float)index;
            }
            if (bn.leaf)
            {
                leaf_fn(bn, fn);
            }
            else
            {
                stack.push_back(FlattenItem{bn.b, index, 1});
                stack.push_back(FlattenItem{bn.a, index, 0});
            }
        }
        return next;
    }
}

int FlattenMesh(const BuiltBvh& bvh, int root_index, int tri_offset, FlatNode* nodes)
{
    return FlattenPreorder(bvh, root_index, nodes, [&](const BuiltNode& bn, FlatNode& fn) {
        fn.LRLeaf.x = (float)(tri_offset + bn.a);
        fn.LRLeaf.y = (float)bn.b;
        fn.LRLeaf.z = 1.f;
    });
}

void FlattenInstances(const BuiltBvh& tlas, int top_index, const int* instance_mesh_root,
                      const int* instance_material, FlatNode* nodes)
{
    FlattenPreorder(tlas, top_index, nodes, [&](const BuiltNode& bn, FlatNode& fn) {
        int inst = tlas.packed[bn.a];
        fn.LRLeaf.x = (float)instance_mesh_root[inst];
        fn.LRLeaf.y = (float)instance_material[inst];
        fn.LRLeaf.z = (float)(-inst - 1);
    });
}
}
