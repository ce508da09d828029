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

/* An 8-wide node of the wide tree that the opt-in fast traversal reads: up to
 * eight children of the binary tree collapsed into one node (the interior
 * child with the largest surface area is replaced by its two children until
 * there are eight or no interior child is left).  Child boxes are stored
 * quantised to 8 bits per plane on a per-node grid p + q * 2^(e - 127), and
 * rounded outwards with one grid step of padding on every side, so a child's
 * quantised box strictly contains its exact box. */
struct WideNode {
    float p[3];
    uint8_t e[3];
    uint8_t nchild;
    uint8_t qlo[3][8], qhi[3][8];   /* [axis][child] */
    int32_t child[8];                /* the child's index in BuildResult.nodes */
    int32_t wchild[8];               /* an interior child's index in WideResult.nodes, -1 for a leaf */
};

struct WideResult {
    std::vector<WideNode> nodes;     /* nodes[0] is the root when the binary root is interior */
    int max_push = 0;                /* most stack entries a traversal can hold below any node */
};

/* collapses the binary tree `br` (interior root) into the wide tree */
WideResult build_wide(const BuildResult& br);

}  // namespace rtb

#endif
