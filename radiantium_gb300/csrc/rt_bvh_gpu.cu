/*
 * rt_bvh_gpu.cu - the reference's SAH tree (rt_bvh.h, Accelerators/Bvh.cs)
 * built on the GPU, level by level.
 *
 * Every level holds the segments (nodes) still to split, each a contiguous
 * range of the item permutation.  Per level:
 *   1. bounds and centroid bounds of every segment (warp-grouped atomics on
 *      order-preserving integer codes of the floats: min / max are exact in
 *      any order);
 *   2. per segment: leaf tests, two-item sort, or the 12 SAH buckets
 *      (counts and bounds gathered like 1), costs, split choice - one thread
 *      with the host builder's operation order;
 *   3. MathExt.Partition reproduced exactly: that two-pointer partition
 *      swaps the k-th item failing the test from the left with the k-th
 *      passing one from the right while the first lies left of the second,
 *      so ranks (two scans) give every destination and the split point;
 *   4. children become the next level's segments (scan over split flags).
 * Finally subtree sizes give the depth-first index of every node and the
 * flattened nodes equal the host builder's.
 */
#include <cuda_runtime.h>
#include <algorithm>
#include <climits>
#include <vector>

#include "rt_bvh.h"
#include "rt_bvh_gpu.h"

namespace {

constexpr int kBuckets = 12;
constexpr float kMaxF = 3.40282347e+38f;

__device__ __forceinline__ int fkey(float f) { const int i = __float_as_int(f); return i >= 0 ? i : i ^ 0x7FFFFFFF; }
__device__ __forceinline__ float fdec(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7FFFFFFF); }

/* (int)float with the x64 .NET semantics of the reference's bucket index */
__device__ __forceinline__ int f2i(float f) {
    if (f != f || f >= 2147483648.0f || f < -2147483648.0f) return INT_MIN;
    return (int)f;
}

struct Seg { int lo, hi, node, pad; };

/* segment accumulators, as order-preserving integer codes */
struct SegAcc {
    int bmin[3], bmax[3];        /* bounds */
    int cmin[3], cmax[3];        /* centroid bounds */
    int cnt[kBuckets];
    int kmin[kBuckets][3], kmax[kBuckets][3];
};

/* per-segment decisions */
struct SegPlan {
    int kind;                    /* 0 leaf, 1 split at mid, 2 SAH buckets pending, 3 partition pending */
    int dim, minb, mid;
};

/* BFS node record */
struct GNode {
    float mn[3], mx[3];
    int left, right;             /* BFS ids of the children (-1: leaf) */
    int lo, count, axis;
};

struct Dev {
    int n = 0;
    const float* box = nullptr;  /* n x 6 */
    float* cent = nullptr;       /* n x 3 */
    int* perm = nullptr; int* perm2 = nullptr;
    int* item_seg = nullptr;     /* active item -> segment of the level, -1 otherwise */
    int* fflag = nullptr; int* tflag = nullptr;   /* n + 1 entries, exclusive scans in place */
    int* fpos = nullptr; int* tpos = nullptr;
    int* bsum = nullptr;         /* block sums of the scans */
    Seg* seg = nullptr; Seg* seg2 = nullptr;
    SegAcc* acc = nullptr;
    SegPlan* plan = nullptr;
    int* split = nullptr;        /* per segment: 2 if split, 0 leaf; scanned */
    GNode* nodes = nullptr;
    int* meta = nullptr;         /* [0] nodes used */
};

__device__ __forceinline__ void box_of(const Dev& D, int id, float* mn, float* mx) {
    const float* b = D.box + (size_t)id * 6;
    mn[0] = b[0]; mn[1] = b[1]; mn[2] = b[2]; mx[0] = b[3]; mx[1] = b[4]; mx[2] = b[5];
}

__global__ void k_init(Dev D) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= D.n) return;
    const float* b = D.box + (size_t)i * 6;
    for (int k = 0; k < 3; k++) D.cent[(size_t)i * 3 + k] = 0.5f * b[k] + 0.5f * b[3 + k];
    D.perm[i] = i;
}

/* segment of every item position (binary search over the level's sorted segments) */
__global__ void k_item_seg(Dev D, int nseg) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < D.n; i += gridDim.x * blockDim.x) {
        int lo = 0, hi = nseg - 1, s = -1;
        while (lo <= hi) {
            const int m = (lo + hi) >> 1;
            if (D.seg[m].lo <= i) { s = m; lo = m + 1; } else hi = m - 1;
        }
        D.item_seg[i] = (s >= 0 && i < D.seg[s].hi) ? s : -1;
    }
}

__global__ void k_acc_reset(Dev D, int nseg) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    SegAcc& a = D.acc[s];
    for (int k = 0; k < 3; k++) {
        a.bmin[k] = a.cmin[k] = fkey(kMaxF); a.bmax[k] = a.cmax[k] = fkey(-kMaxF);
    }
    for (int b = 0; b < kBuckets; b++) {
        a.cnt[b] = 0;
        for (int k = 0; k < 3; k++) { a.kmin[b][k] = fkey(kMaxF); a.kmax[b][k] = fkey(-kMaxF); }
    }
}

/* min / max of a value over the lanes sharing `peers`, then one atomic */
__device__ __forceinline__ void grp_min(unsigned peers, int leader, int lane, int v, int* dst) {
    const int r = (int)__reduce_min_sync(peers, (unsigned)(v ^ INT_MIN)) ^ INT_MIN;
    if (lane == leader) atomicMin(dst, r);
}
__device__ __forceinline__ void grp_max(unsigned peers, int leader, int lane, int v, int* dst) {
    const int r = (int)__reduce_max_sync(peers, (unsigned)(v ^ INT_MIN)) ^ INT_MIN;
    if (lane == leader) atomicMax(dst, r);
}

__global__ void k_bounds(Dev D) {
    const int lane = threadIdx.x & 31;
    for (int i0 = blockIdx.x * blockDim.x; i0 < D.n; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + threadIdx.x;
        const int s = i < D.n ? D.item_seg[i] : -1;
        const unsigned act = __ballot_sync(0xffffffffu, s >= 0);
        if (s < 0) continue;
        const unsigned peers = __match_any_sync(act, s);
        const int leader = __ffs(peers) - 1;
        const int id = D.perm[i];
        float mn[3], mx[3];
        box_of(D, id, mn, mx);
        SegAcc& a = D.acc[s];
        for (int k = 0; k < 3; k++) {
            const float c = D.cent[(size_t)id * 3 + k];
            grp_min(peers, leader, lane, fkey(mn[k]), &a.bmin[k]);
            grp_max(peers, leader, lane, fkey(mx[k]), &a.bmax[k]);
            grp_min(peers, leader, lane, fkey(c), &a.cmin[k]);
            grp_max(peers, leader, lane, fkey(c), &a.cmax[k]);
        }
    }
}

/* bucket of a centroid along dim (BoundingBox3F.Offset, then (int)(12 * o)) */
__device__ __forceinline__ int bucket_of(const float* cmn, const float* cmx, int dim, float c) {
    float o = c - cmn[dim];
    if (cmx[dim] > cmn[dim]) o /= cmx[dim] - cmn[dim];
    return f2i(12.0f * o);
}
__device__ __forceinline__ void dec_cb(const SegAcc& a, float* cmn, float* cmx) {
    for (int k = 0; k < 3; k++) { cmn[k] = fdec(a.cmin[k]); cmx[k] = fdec(a.cmax[k]); }
}
__device__ __forceinline__ int maximum_extent(const float* mn, const float* mx) {
    const float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
    if (dx > dy && dx > dz) return 0;
    if (dy > dz) return 1;
    return 2;
}
__device__ __forceinline__ float surface_area(const float* mn, const float* mx) {
    const float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
    return 2 * (dx * dy + dx * dz + dy * dz);
}

/* 2: leaf tests, the two-item sort, or the SAH bucket pass */
__global__ void k_plan1(Dev D, int nseg, int level_base) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const Seg g = D.seg[s];
    const SegAcc& a = D.acc[s];
    GNode& nd = D.nodes[g.node];
    for (int k = 0; k < 3; k++) { nd.mn[k] = fdec(a.bmin[k]); nd.mx[k] = fdec(a.bmax[k]); }
    nd.left = nd.right = -1; nd.lo = g.lo; nd.count = g.hi - g.lo; nd.axis = 0;
    SegPlan p{0, 0, 0, 0};
    const int n = g.hi - g.lo;
    if (n > 1) {
        float cmn[3], cmx[3];
        dec_cb(a, cmn, cmx);
        const int dim = maximum_extent(cmn, cmx);
        p.dim = dim;
        if (cmx[dim] == cmn[dim]) {
            p.kind = 0;
        } else if (n <= 2) {
            const int i0 = D.perm[g.lo], i1 = D.perm[g.lo + 1];
            const float lv = D.cent[(size_t)i0 * 3 + dim], rv = D.cent[(size_t)i1 * 3 + dim];
            const int cmp = (lv == rv) ? 0 : (lv < rv ? -1 : 1);
            if (cmp > 0) { D.perm[g.lo] = i1; D.perm[g.lo + 1] = i0; }
            p.kind = 1;
            p.mid = (g.lo + g.hi) / 2;
        } else {
            p.kind = 2;
        }
    }
    D.plan[s] = p;
}

__global__ void k_buckets(Dev D) {
    const int lane = threadIdx.x & 31;
    for (int i0 = blockIdx.x * blockDim.x; i0 < D.n; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + threadIdx.x;
        int s = i < D.n ? D.item_seg[i] : -1;
        if (s >= 0 && D.plan[s].kind != 2) s = -1;
        const unsigned act = __ballot_sync(0xffffffffu, s >= 0);
        if (s < 0) continue;
        const SegAcc& a = D.acc[s];
        float cmn[3], cmx[3];
        dec_cb(a, cmn, cmx);
        const int dim = D.plan[s].dim;
        const int id = D.perm[i];
        int b = bucket_of(cmn, cmx, dim, D.cent[(size_t)id * 3 + dim]);
        if (b == kBuckets) b = kBuckets - 1;
        if (b < 0 || b > kBuckets - 1) b = b < 0 ? 0 : kBuckets - 1;
        const unsigned peers = __match_any_sync(act, s * kBuckets + b);
        const int leader = __ffs(peers) - 1;
        float mn[3], mx[3];
        box_of(D, id, mn, mx);
        SegAcc& w = D.acc[s];
        if (lane == leader) atomicAdd(&w.cnt[b], __popc(peers));
        for (int k = 0; k < 3; k++) {
            grp_min(peers, leader, lane, fkey(mn[k]), &w.kmin[b][k]);
            grp_max(peers, leader, lane, fkey(mx[k]), &w.kmax[b][k]);
        }
    }
}

/* SAH costs in the host builder's order; leaf or partition */
__global__ void k_plan2(Dev D, int nseg, int max_prims) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg || D.plan[s].kind != 2) return;
    const Seg g = D.seg[s];
    const SegAcc& a = D.acc[s];
    const int n = g.hi - g.lo;
    float bmn[3], bmx[3];
    for (int k = 0; k < 3; k++) { bmn[k] = fdec(a.bmin[k]); bmx[k] = fdec(a.bmax[k]); }
    float cost[kBuckets - 1];
    for (int sp = 0; sp < kBuckets - 1; sp++) {
        float b0n[3] = {kMaxF, kMaxF, kMaxF}, b0x[3] = {-kMaxF, -kMaxF, -kMaxF};
        float b1n[3] = {kMaxF, kMaxF, kMaxF}, b1x[3] = {-kMaxF, -kMaxF, -kMaxF};
        int c0 = 0, c1 = 0;
        for (int j = 0; j <= sp; j++) {
            for (int k = 0; k < 3; k++) {
                const float qn = fdec(a.kmin[j][k]), qx = fdec(a.kmax[j][k]);
                b0n[k] = b0n[k] < qn ? b0n[k] : qn;
                b0x[k] = b0x[k] > qx ? b0x[k] : qx;
            }
            c0 += a.cnt[j];
        }
        for (int j = sp + 1; j < kBuckets; j++) {
            for (int k = 0; k < 3; k++) {
                const float qn = fdec(a.kmin[j][k]), qx = fdec(a.kmax[j][k]);
                b1n[k] = b1n[k] < qn ? b1n[k] : qn;
                b1x[k] = b1x[k] > qx ? b1x[k] : qx;
            }
            c1 += a.cnt[j];
        }
        cost[sp] = 1 + ((float)c0 * surface_area(b0n, b0x) + (float)c1 * surface_area(b1n, b1x)) / surface_area(bmn, bmx);
    }
    float min_cost = cost[0];
    int min_b = 0;
    for (int sp = 1; sp < kBuckets - 1; sp++) if (cost[sp] < min_cost) { min_cost = cost[sp]; min_b = sp; }
    SegPlan p = D.plan[s];
    if (n > max_prims || min_cost < (float)n) { p.kind = 3; p.minb = min_b; }
    else p.kind = 0;
    D.plan[s] = p;
}

/* partition test per item (raw bucket index, as the host builder's lambda) */
__global__ void k_part_flags(Dev D) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < D.n; i += gridDim.x * blockDim.x) {
        const int s = D.item_seg[i];
        int f = 0, t = 0;
        if (s >= 0 && D.plan[s].kind == 3) {
            float cmn[3], cmx[3];
            dec_cb(D.acc[s], cmn, cmx);
            const SegPlan p = D.plan[s];
            const int id = D.perm[i];
            const bool pred = bucket_of(cmn, cmx, p.dim, D.cent[(size_t)id * 3 + p.dim]) <= p.minb;
            t = pred ? 1 : 0;
            f = pred ? 0 : 1;
        }
        D.fflag[i] = f;
        D.tflag[i] = t;
    }
}

/* exclusive scan of n ints in place (a[n] receives the total): block scans,
 * a single-block scan of the block sums, then the offsets */
__global__ void k_scan_block(int* a, int n, int* bsum) {
    __shared__ int sh[1024];
    const int i = blockIdx.x * 1024 + threadIdx.x;
    const int v = i < n ? a[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        const int t = threadIdx.x >= (unsigned)off ? sh[threadIdx.x - off] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) a[i] = sh[threadIdx.x] - v;
    if (threadIdx.x == 1023) bsum[blockIdx.x] = sh[1023];
}
__global__ void k_scan_sums(int* bsum, int nb) {
    __shared__ int carry;
    __shared__ int sh[1024];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int base = 0; base < nb; base += 1024) {
        const int i = base + threadIdx.x;
        const int v = i < nb ? bsum[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < 1024; off <<= 1) {
            const int t = threadIdx.x >= (unsigned)off ? sh[threadIdx.x - off] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) bsum[i] = carry + sh[threadIdx.x] - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry += sh[1023];
        __syncthreads();
    }
    if (threadIdx.x == 0) bsum[nb] = carry;
}
__global__ void k_scan_add(int* a, int n, const int* bsum, int nb) {
    const int i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n) a[i] += bsum[blockIdx.x];
    if (i == 0) a[n] = bsum[nb];
}

/* ranks: the k-th failing item from the left, the k-th passing one from the right */
__global__ void k_part_ranks(Dev D) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < D.n; i += gridDim.x * blockDim.x) {
        const int s = D.item_seg[i];
        if (s < 0 || D.plan[s].kind != 3) continue;
        const Seg g = D.seg[s];
        const bool fail = D.fflag[i + 1] - D.fflag[i] == 1;
        if (fail) {
            D.fpos[g.lo + (D.fflag[i] - D.fflag[g.lo])] = i;
        } else {
            const int tcount = D.tflag[g.hi] - D.tflag[g.lo];
            const int before = D.tflag[i + 1] - D.tflag[g.lo];      /* passing items in [lo, i] */
            D.tpos[g.lo + (tcount - before)] = i;
        }
    }
}

/* swaps K and the split point of MathExt.Partition(list, lo, hi - 1) */
__global__ void k_part_k(Dev D, int nseg) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg || D.plan[s].kind != 3) return;
    const Seg g = D.seg[s];
    const int nf = D.fflag[g.hi] - D.fflag[g.lo], nt = D.tflag[g.hi] - D.tflag[g.lo];
    int lo = 0, hi = min(nf, nt);                     /* largest K with fpos[K-1] < tpos[K-1] */
    while (lo < hi) {
        const int m = (lo + hi + 1) >> 1;
        if (D.fpos[g.lo + m - 1] < D.tpos[g.lo + m - 1]) lo = m; else hi = m - 1;
    }
    const int K = lo;
    const int tK = K == 0 ? g.hi - 1 : D.tpos[g.lo + K - 1];
    int mid = tK;
    if (K < nf && D.fpos[g.lo + K] < tK) mid = D.fpos[g.lo + K];
    SegPlan p = D.plan[s];
    p.mid = mid;
    p.minb = K;                                       /* reused: swaps count for k_part_move */
    D.plan[s] = p;
}

__global__ void k_part_move(Dev D) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < D.n; i += gridDim.x * blockDim.x) {
        const int s = D.item_seg[i];
        int dst = i;
        if (s >= 0 && D.plan[s].kind == 3) {
            const Seg g = D.seg[s];
            const int K = D.plan[s].minb;
            const bool fail = D.fflag[i + 1] - D.fflag[i] == 1;
            if (fail) {
                const int r = D.fflag[i] - D.fflag[g.lo];
                if (r < K) dst = D.tpos[g.lo + r];
            } else {
                const int r = (D.tflag[g.hi] - D.tflag[g.lo]) - (D.tflag[i + 1] - D.tflag[g.lo]);
                if (r < K) dst = D.fpos[g.lo + r];
            }
        }
        D.perm2[dst] = D.perm[i];
    }
}

/* split flags for the children scan */
__global__ void k_split_flags(Dev D, int nseg) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < nseg) D.split[s] = (D.plan[s].kind == 1 || D.plan[s].kind == 3) ? 2 : 0;
}

/* children of every split segment, in segment order (so sorted by lo) */
__global__ void k_children(Dev D, int nseg, int next_node_base) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nseg) return;
    const SegPlan p = D.plan[s];
    if (!(p.kind == 1 || p.kind == 3)) return;
    const Seg g = D.seg[s];
    const int o = D.split[s];
    const int ln = next_node_base + o, rn = next_node_base + o + 1;
    D.seg2[o] = Seg{g.lo, p.mid, ln, 0};
    D.seg2[o + 1] = Seg{p.mid, g.hi, rn, 0};
    GNode& nd = D.nodes[g.node];
    nd.left = ln; nd.right = rn; nd.count = 0; nd.axis = p.dim;
}

inline unsigned gridn(long long n, int b) { return (unsigned)std::max<long long>(1, (n + b - 1) / b); }

void scan(int* a, int n, int* bsum, cudaStream_t s) {
    const int nb = (n + 1023) / 1024;
    k_scan_block<<<nb, 1024, 0, s>>>(a, n, bsum);
    k_scan_sums<<<1, 1024, 0, s>>>(bsum, nb);
    k_scan_add<<<nb, 1024, 0, s>>>(a, n, bsum, nb);
}

}  // namespace

#define GK(x) do { cudaError_t e_ = (x); if (e_ != cudaSuccess) { err = e_; goto done; } } while (0)

cudaError_t rt_gpu_build_sah(const std::vector<rtb::Box>& bounds, int max_prims, rtb::BuildResult* out,
                             cudaStream_t s) {
    cudaError_t err = cudaSuccess;
    const int n = (int)bounds.size();
    *out = rtb::BuildResult();
    if (n == 0) return cudaSuccess;
    if (max_prims < 1) max_prims = 1;
    Dev D;
    D.n = n;
    float* d_box = nullptr;
    std::vector<GNode> hn;
    std::vector<int> perm;
    std::vector<int> level_start;       /* first BFS node id of every level */
    int nodes_used = 1, nseg = 1;
    const int max_nodes = 2 * n;
    const int nbs = (n + 1023) / 1024 + 2;
    GK(rt_dev_malloc((void**)&d_box, (size_t)n * 6 * sizeof(float)));
    GK(cudaMemcpyAsync(d_box, bounds.data(), (size_t)n * 6 * sizeof(float), cudaMemcpyHostToDevice, s));
    D.box = d_box;
    GK(rt_dev_malloc((void**)&D.cent, (size_t)n * 3 * sizeof(float)));
    GK(rt_dev_malloc((void**)&D.perm, (size_t)n * sizeof(int)));
    GK(rt_dev_malloc((void**)&D.perm2, (size_t)n * sizeof(int)));
    GK(rt_dev_malloc((void**)&D.item_seg, (size_t)n * sizeof(int)));
    GK(rt_dev_malloc((void**)&D.fflag, (size_t)(n + 1) * sizeof(int)));
    GK(rt_dev_malloc((void**)&D.tflag, (size_t)(n + 1) * sizeof(int)));
    GK(rt_dev_malloc((void**)&D.fpos, (size_t)n * sizeof(int)));
    GK(rt_dev_malloc((void**)&D.tpos, (size_t)n * sizeof(int)));
    GK(rt_dev_malloc((void**)&D.bsum, (size_t)nbs * sizeof(int)));
    GK(rt_dev_malloc((void**)&D.seg, (size_t)n * sizeof(Seg)));
    GK(rt_dev_malloc((void**)&D.seg2, (size_t)n * sizeof(Seg)));
    GK(rt_dev_malloc((void**)&D.acc, (size_t)n * sizeof(SegAcc)));
    GK(rt_dev_malloc((void**)&D.plan, (size_t)n * sizeof(SegPlan)));
    GK(rt_dev_malloc((void**)&D.split, (size_t)(n + 1) * sizeof(int)));
    GK(rt_dev_malloc((void**)&D.nodes, (size_t)max_nodes * sizeof(GNode)));
    k_init<<<gridn(n, 256), 256, 0, s>>>(D);
    {
        const Seg root{0, n, 0, 0};
        GK(cudaMemcpyAsync(D.seg, &root, sizeof(Seg), cudaMemcpyHostToDevice, s));
    }
    level_start.push_back(0);
    while (nseg > 0) {
        const unsigned gi = std::min(gridn(n, 256), 152u * 16u);
        k_item_seg<<<gi, 256, 0, s>>>(D, nseg);
        k_acc_reset<<<gridn(nseg, 128), 128, 0, s>>>(D, nseg);
        k_bounds<<<gi, 256, 0, s>>>(D);
        k_plan1<<<gridn(nseg, 128), 128, 0, s>>>(D, nseg, 0);
        k_buckets<<<gi, 256, 0, s>>>(D);
        k_plan2<<<gridn(nseg, 128), 128, 0, s>>>(D, nseg, max_prims);
        k_part_flags<<<gi, 256, 0, s>>>(D);
        scan(D.fflag, n, D.bsum, s);
        scan(D.tflag, n, D.bsum, s);
        k_part_ranks<<<gi, 256, 0, s>>>(D);
        k_part_k<<<gridn(nseg, 128), 128, 0, s>>>(D, nseg);
        k_part_move<<<gi, 256, 0, s>>>(D);
        std::swap(D.perm, D.perm2);
        k_split_flags<<<gridn(nseg, 256), 256, 0, s>>>(D, nseg);
        scan(D.split, nseg, D.bsum, s);
        int next = 0;
        GK(cudaMemcpyAsync(&next, D.split + nseg, sizeof(int), cudaMemcpyDeviceToHost, s));
        GK(cudaStreamSynchronize(s));
        GK(cudaGetLastError());
        if (nodes_used + next > max_nodes) { err = cudaErrorInvalidValue; goto done; }
        k_children<<<gridn(nseg, 128), 128, 0, s>>>(D, nseg, nodes_used);
        std::swap(D.seg, D.seg2);
        level_start.push_back(nodes_used);
        nodes_used += next;
        nseg = next;
    }
    /* depth-first flattening on the host from the BFS records */
    hn.resize(nodes_used);
    perm.resize(n);
    GK(cudaMemcpyAsync(hn.data(), D.nodes, (size_t)nodes_used * sizeof(GNode), cudaMemcpyDeviceToHost, s));
    GK(cudaMemcpyAsync(perm.data(), D.perm, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost, s));
    GK(cudaStreamSynchronize(s));
    GK(cudaGetLastError());
    {
        std::vector<int> size(nodes_used, 1), dfs(nodes_used, 0);
        for (int v = nodes_used - 1; v >= 0; v--)
            if (hn[v].left >= 0) size[v] = 1 + size[hn[v].left] + size[hn[v].right];
        for (int v = 0; v < nodes_used; v++)         /* BFS order: parents before children */
            if (hn[v].left >= 0) {
                dfs[hn[v].left] = dfs[v] + 1;
                dfs[hn[v].right] = dfs[v] + 1 + size[hn[v].left];
            }
        out->nodes.resize(nodes_used);
        for (int v = 0; v < nodes_used; v++) {
            rtb::FlatNode& f = out->nodes[dfs[v]];
            for (int k = 0; k < 3; k++) { f.bounds.mn[k] = hn[v].mn[k]; f.bounds.mx[k] = hn[v].mx[k]; }
            if (hn[v].left >= 0) { f.second = dfs[hn[v].right]; f.count = 0; f.axis = hn[v].axis; }
            else { f.second = hn[v].lo; f.count = hn[v].count; f.axis = 0; }
        }
        out->order.assign(perm.begin(), perm.end());
        out->max_depth = (int)level_start.size() - 1;
    }
done:
    cudaFree(d_box); cudaFree(D.cent); cudaFree(D.perm); cudaFree(D.perm2); cudaFree(D.item_seg);
    cudaFree(D.fflag); cudaFree(D.tflag); cudaFree(D.fpos); cudaFree(D.tpos); cudaFree(D.bsum);
    cudaFree(D.seg); cudaFree(D.seg2); cudaFree(D.acc); cudaFree(D.plan); cudaFree(D.split); cudaFree(D.nodes);
    return err;
}
