/*
 * rt_bvh.cpp - SAH BVH construction producing the reference's tree
 * (see rt_bvh.h).  Compiled with -ffp-contract=off: every bucket cost and
 * centroid offset must round like the reference's single-precision code.
 */
#include "rt_bvh.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <future>
#include <limits.h>
#include <utility>

namespace rtb {

static const float kMax = 3.40282347e+38f;

Box empty_box() {
    Box b;
    for (int i = 0; i < 3; i++) { b.mn[i] = kMax; b.mx[i] = -kMax; }
    return b;
}
/* Vector3.Min / Max element-wise: (a < b ? a : b), (a > b ? a : b) */
void box_union(Box& a, const Box& b) {
    for (int i = 0; i < 3; i++) {
        a.mn[i] = a.mn[i] < b.mn[i] ? a.mn[i] : b.mn[i];
        a.mx[i] = a.mx[i] > b.mx[i] ? a.mx[i] : b.mx[i];
    }
}
void box_expand(Box& a, const float* p) {
    for (int i = 0; i < 3; i++) {
        a.mn[i] = a.mn[i] < p[i] ? a.mn[i] : p[i];
        a.mx[i] = a.mx[i] > p[i] ? a.mx[i] : p[i];
    }
}
static inline float surface_area(const Box& b) {
    float dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
    return 2 * (dx * dy + dx * dz + dy * dz);
}
static inline int maximum_extent(const Box& b) {
    float dx = b.mx[0] - b.mn[0], dy = b.mx[1] - b.mn[1], dz = b.mx[2] - b.mn[2];
    if (dx > dy && dx > dz) return 0;
    if (dy > dz) return 1;
    return 2;
}
/* (int)float with the x64 .NET semantics used by the reference's bucket index */
static inline int f2i(float f) {
    if (f != f || f >= 2147483648.0f || f < -2147483648.0f) return INT_MIN;
    return (int)f;
}

namespace {

struct Item {
    Box b;
    float c[3];
    int32_t id;
};

class Builder {
public:
    Builder(std::vector<Item>& it, int max_prims, int par_depth) : items_(it), max_prims_(max_prims), par_depth_(par_depth) {}

    /* bucket of a centroid along dim (BoundingBox3F.Offset, then (int)(12 * o)) */
    static inline int bucket_of(const Box& cb, int dim, const float* c) {
        float o = c[dim] - cb.mn[dim];
        if (cb.mx[dim] > cb.mn[dim]) o /= cb.mx[dim] - cb.mn[dim];
        return f2i(12.0f * o);
    }

    /* MathExt.Partition(list, lo, last) with `last` inclusive */
    template <class Pred>
    int partition(int lo, int last, Pred pred) {
        int first = lo;
        while (true) {
            while (true) {
                if (first == last) return first;
                if (!pred(items_[first])) break;
                ++first;
            }
            while (!pred(items_[last])) {
                if (first == last) return first;
                last--;
            }
            std::swap(items_[first], items_[last]);
            first++;
        }
    }

    /* appends the subtree of items [lo, hi) to `out` in depth-first order;
     * right-child indices are relative to the start of `out` */
    int build(std::vector<FlatNode>& out, int lo, int hi, int level) {
        Box bounds = empty_box();
        for (int i = lo; i < hi; i++) box_union(bounds, items_[i].b);
        const int n = hi - lo;
        const int idx = (int)out.size();
        FlatNode leafn;
        leafn.bounds = bounds; leafn.second = lo; leafn.count = n; leafn.axis = 0;
        if (n == 1) { out.push_back(leafn); return 1; }
        Box cb = empty_box();
        for (int i = lo; i < hi; i++) box_expand(cb, items_[i].c);
        const int dim = maximum_extent(cb);
        int mid = (lo + hi) / 2;
        if (cb.mx[dim] == cb.mn[dim]) { out.push_back(leafn); return 1; }
        if (n <= 2) {
            float lv = items_[lo].c[dim], rv = items_[lo + 1].c[dim];
            int cmp = (lv == rv) ? 0 : (lv < rv ? -1 : 1);
            if (cmp > 0) std::swap(items_[lo], items_[lo + 1]);
        } else {
            const int NB = 12;
            int count[NB] = {0};
            Box bb[NB];
            for (int i = 0; i < NB; i++) bb[i] = empty_box();
            for (int i = lo; i < hi; i++) {
                int b = bucket_of(cb, dim, items_[i].c);
                if (b == NB) b = NB - 1;
                if (b < 0 || b > NB - 1) b = b < 0 ? 0 : NB - 1; /* unreachable for finite centroids */
                count[b]++;
                box_union(bb[b], items_[i].b);
            }
            /* split costs with the reference's per-split union loops (same union order) */
            float cost[NB - 1];
            for (int s = 0; s < NB - 1; s++) {
                Box b0 = empty_box(), b1 = empty_box();
                int c0 = 0, c1 = 0;
                for (int j = 0; j <= s; j++) { box_union(b0, bb[j]); c0 += count[j]; }
                for (int j = s + 1; j < NB; j++) { box_union(b1, bb[j]); c1 += count[j]; }
                cost[s] = 1 + ((float)c0 * surface_area(b0) + (float)c1 * surface_area(b1)) / surface_area(bounds);
            }
            float min_cost = cost[0];
            int min_b = 0;
            for (int s = 1; s < NB - 1; s++) if (cost[s] < min_cost) { min_cost = cost[s]; min_b = s; }
            if (n > max_prims_ || min_cost < (float)n) {
                mid = partition(lo, hi - 1, [&](const Item& it) { return bucket_of(cb, dim, it.c) <= min_b; });
            } else {
                out.push_back(leafn);
                return 1;
            }
        }
        FlatNode node;
        node.count = 0;
        node.axis = dim;
        out.push_back(node);
        int dl, dr;
        if (level < par_depth_ && n > 65536) {
            std::vector<FlatNode> left, right;
            auto fut = std::async(std::launch::async, [&]() { return build(left, lo, mid, level + 1); });
            dr = build(right, mid, hi, level + 1);
            dl = fut.get();
            splice(out, left);
            out[idx].second = (int)out.size();
            splice(out, right);
        } else {
            dl = build(out, lo, mid, level + 1);
            out[idx].second = (int)out.size();
            dr = build(out, mid, hi, level + 1);
        }
        Box nb = out[idx + 1].bounds;
        box_union(nb, out[out[idx].second].bounds);
        out[idx].bounds = nb;
        return 1 + std::max(dl, dr);
    }

private:
    static void splice(std::vector<FlatNode>& out, std::vector<FlatNode>& s) {
        const int base = (int)out.size();
        for (FlatNode& n : s) {
            if (n.count == 0) n.second += base;
            out.push_back(n);
        }
        std::vector<FlatNode>().swap(s);
    }
    std::vector<Item>& items_;
    int max_prims_;
    int par_depth_;
};

}  // namespace

BuildResult build_sah(const std::vector<Box>& prim_bounds, int max_prims, int threads) {
    BuildResult r;
    const int n = (int)prim_bounds.size();
    if (n == 0) return r;
    std::vector<Item> items(n);
    for (int i = 0; i < n; i++) {
        items[i].b = prim_bounds[i];
        for (int k = 0; k < 3; k++) items[i].c[k] = 0.5f * prim_bounds[i].mn[k] + 0.5f * prim_bounds[i].mx[k];
        items[i].id = i;
    }
    int par_depth = 0;
    while ((1 << par_depth) < threads && par_depth < 6) par_depth++;
    Builder b(items, max_prims < 1 ? 1 : max_prims, par_depth);
    r.nodes.reserve(2 * (size_t)n);
    r.max_depth = b.build(r.nodes, 0, n, 0);
    r.order.resize(n);
    for (int i = 0; i < n; i++) r.order[i] = items[i].id;
    return r;
}

/* ---- the wide tree of the fast traversal -------------------------------------------------- */

/* The quantisation grid of one axis of a node box [mn, mx]: scale 2^k with k
 * large enough that 253 steps cover the extent and that one step is at least
 * 2^-20 of the coordinates' magnitude (so the one-step padding outweighs the
 * rounding of the traversal's plane distances), origin one step below mn
 * (rounded down).  Children are quantised outwards with one more step of
 * padding; k grows until every child fits in [0, 255]. */
static void quantise_axis(double mn, double mx, const std::vector<std::pair<double, double>>& kids, float* p,
                          uint8_t* e, uint8_t* qlo, uint8_t* qhi) {
    const double ext = mx - mn;
    const double mag = std::max(std::max(std::fabs(mn), std::fabs(mx)), 1e-30);
    int k = std::max(ext > 0 ? (int)std::ceil(std::log2(ext / 253.0)) : -126, (int)std::floor(std::log2(mag)) - 20);
    for (k = std::max(k, -126); k <= 127; k++) {
        const double s = std::ldexp(1.0, k);
        float pf = (float)(mn - s);
        if ((double)pf > mn - s) pf = std::nextafter(pf, -INFINITY);
        bool ok = std::isfinite(pf);
        int lo[8] = {0}, hi[8] = {0};
        for (size_t c = 0; ok && c < kids.size(); c++) {
            lo[c] = (int)std::floor((kids[c].first - (double)pf) / s) - 1;
            hi[c] = (int)std::ceil((kids[c].second - (double)pf) / s) + 1;
            ok = lo[c] >= 0 && hi[c] <= 255;
        }
        if (!ok) continue;
        *p = pf;
        *e = (uint8_t)(k + 127);
        for (size_t c = 0; c < 8; c++) {
            qlo[c] = c < kids.size() ? (uint8_t)lo[c] : 255;    /* empty slots: lo > hi, never hit */
            qhi[c] = c < kids.size() ? (uint8_t)hi[c] : 0;
        }
        return;
    }
    *p = (float)mn; *e = 254;                                     /* unreachable for finite boxes */
    for (int c = 0; c < 8; c++) { qlo[c] = 0; qhi[c] = 255; }
}

WideResult build_wide(const BuildResult& br) {
    WideResult r;
    const std::vector<FlatNode>& fn = br.nodes;
    if (fn.empty() || fn[0].count != 0) return r;
    struct Work { int bnode, wnode, push; };
    std::vector<Work> work{{0, 0, 0}};
    r.nodes.emplace_back();
    while (!work.empty()) {
        const Work w = work.back();
        work.pop_back();
        std::vector<int> kids{w.bnode + 1, fn[w.bnode].second};
        while (kids.size() < 8) {
            int best = -1;
            float best_a = -1.0f;
            for (size_t i = 0; i < kids.size(); i++) {
                if (fn[kids[i]].count != 0) continue;
                const float a = surface_area(fn[kids[i]].bounds);
                if (a > best_a) { best_a = a; best = (int)i; }
            }
            if (best < 0) break;
            const int b = kids[best];
            kids[best] = b + 1;
            kids.insert(kids.begin() + best + 1, fn[b].second);
        }
        WideNode& n = r.nodes[w.wnode];
        std::memset(&n, 0, sizeof(n));
        n.nchild = (uint8_t)kids.size();
        const Box& nb = fn[w.bnode].bounds;
        for (int a = 0; a < 3; a++) {
            std::vector<std::pair<double, double>> iv;
            for (int k : kids) iv.emplace_back((double)fn[k].bounds.mn[a], (double)fn[k].bounds.mx[a]);
            quantise_axis((double)nb.mn[a], (double)nb.mx[a], iv, &n.p[a], &n.e[a], n.qlo[a], n.qhi[a]);
        }
        const int push = w.push + (int)kids.size() - 1;
        r.max_push = std::max(r.max_push, w.push);
        for (size_t i = 0; i < 8; i++) {
            n.child[i] = i < kids.size() ? kids[i] : -1;
            n.wchild[i] = -1;
        }
        for (size_t i = 0; i < kids.size(); i++) {
            if (fn[kids[i]].count != 0) continue;
            const int wi = (int)r.nodes.size();
            r.nodes[w.wnode].wchild[i] = wi;     /* r.nodes may reallocate below: index, not the reference */
            r.nodes.emplace_back();
            work.push_back({kids[i], wi, push});
        }
    }
    return r;
}

}  // namespace rtb
