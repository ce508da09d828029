/*
 * rt_bvh.h - SAH BVH construction producing the reference's tree.
 *
 * The tree must be the one Accelerators/Bvh.cs builds (12-bucket SAH over
 * centroid bounds, split axis = BoundingBox3F.MaximumExtent, MathExt.Partition
 * semantics, two-primitive nodes sorted by centroid, depth-first flattening)
 * because closest-hit ties are resolved by traversal order.  The builder below
 * is an array-based, multi-threaded implementation of that algorithm: the two
 * subtrees of every large node are built concurrently and then spliced in
 * depth-first order.
 */
#ifndef RT_BVH_H
#define RT_BVH_H

#include <stdint.h>
#include <vector>

namespace rtb {

struct Box {
    float mn[3], mx[3];
};
Box empty_box();
void box_union(Box& a, const Box& b);
void box_expand(Box& a, const float* p);

/* one flattened node in depth-first order, as LinearBVHNode */
struct FlatNode {
    Box bounds;
    int32_t second;   /* interior: index of the right child; leaf: first primitive slot */
    int32_t count;    /* 0: interior */
    int32_t axis;
};

struct BuildResult {
    std::vector<FlatNode> nodes;
    std::vector<int32_t> order;   /* slot -> primitive index */
    int max_depth = 0;
};

/* prim_bounds: n boxes in primitive-list order */
BuildResult build_sah(const std::vector<Box>& prim_bounds, int max_prims, int threads);

}  // namespace rtb

#endif
