/*
 * or_scene.cpp - CPU oracle, part 3: shapes, BVH, materials, lights, media,
 * camera, scene services and the scene builder.
 *
 * TEST INFRASTRUCTURE ONLY (see or_core.h).  Each function follows the C#
 * source named beside it, operation by operation.
 */
#include <algorithm>
#include <string>
#include <cmath>
#include "or_scene.h"

namespace orc {

thread_local Counters* tl_counters = nullptr;
static inline void cnt_node() { if (tl_counters) tl_counters->node_visits++; }
static inline void cnt_prim() { if (tl_counters) tl_counters->prim_tests++; }
static inline void cnt_inst() { if (tl_counters) tl_counters->instance_visits++; }

/* ---- Intersection helpers (Intersection.cs:27-71) ----------------------------- */
bool Intersection::IsLight() const { return Shape->GetLight() != nullptr; }
const AreaLight* Intersection::Light() const { return Shape->GetLight(); }
bool Intersection::HasSurface() const { return Shape->GetMaterial() != nullptr; }
const Material* Intersection::Surface() const { return Shape->GetMaterial(); }
C3 Intersection::Le(V3 w) const { const AreaLight* l = Shape->GetLight(); return l == nullptr ? c3s(0.0f) : l->L(*this, w); }
const Medium* Intersection::GetMedium(V3 w) const {
    const MediumAdapter* m = Shape->GetMedium();
    return Dot(w, N()) > 0 ? m->Outside : m->Inside;
}

/* ---- TextureSampler.Sample (TextureSampler.cs:28-72) -------------------------- */
static inline float Wrapper(float a, int mode) {
    if (mode == RT_WRAP_CLAMP) return netClamp(a, 0, 1);
    return netClamp(a - floorf(a), 0, 1);
}
C3 Texture2D::Sample(float x, float y) const {
    float u = Wrapper(x, Wrap);
    float v = Wrapper(y, Wrap);
    int width = Width, height = Height;
    float fu = u * (float)(width - 1);
    float fv = v * (float)(height - 1);
    int pu = netF2I(fu);
    int pv = netF2I(fv);
    if (Filter == RT_FILTER_LINEAR) {
        int dpu = (fu > (float)pu + 0.5f) ? 1 : -1;
        int dpv = (fv > (float)pv + 0.5f) ? 1 : -1;
        int apu = netClampI(pu + dpu, 0, width - 1);
        int apv = netClampI(pv + dpv, 0, height - 1);
        float du = netMin(Abs(fu - (float)pu - 0.5f), 1);
        float dv = netMin(Abs(fv - (float)pv - 0.5f), 1);
        C3 u0v0 = Read(pu, pv), u1v0 = Read(apu, pv), u0v1 = Read(pu, apv), u1v1 = Read(apu, apv);
        return (u0v0 * (1 - du) + u1v0 * du) * (1 - dv) + (u0v1 * (1 - du) + u1v1 * du) * dv;
    }
    return Read(pu, pv);
}

/* ---- Triangle (Shapes/Triangle.cs:65-213) ------------------------------------- */
Triangle::Triangle(const TriangleMesh* m, int i) : Mesh(m), Index(i) {
    BBox b(Pa()); b.ExpendBy(Pb()); b.ExpendBy(Pc());
    WorldBound = b;
    Area = 0.5f * Length(Cross(Pb() - Pa(), Pc() - Pa()));
}
static inline void TriBaryAttrs(const Triangle& tr, V3 bary, V3* p, V3* n, V2* uv) {
    *p = bary.x * tr.Pa() + bary.y * tr.Pb() + bary.z * tr.Pc();
    const TriangleMesh* M = tr.Mesh;
    int i0 = M->Indices[tr.Index * 3 + 0], i1 = M->Indices[tr.Index * 3 + 1], i2 = M->Indices[tr.Index * 3 + 2];
    if (M->HasNormal()) *n = Normalize(bary.x * M->Normal[i0] + bary.y * M->Normal[i1] + bary.z * M->Normal[i2]);
    else *n = Normalize(Cross(tr.Pb() - tr.Pa(), tr.Pc() - tr.Pa()));
    if (M->HasUV()) *uv = bary.x * M->UV[i0] + bary.y * M->UV[i1] + bary.z * M->UV[i2];
    else *uv = bary.x * v2(0, 0) + bary.y * v2(1, 0) + bary.z * v2(1, 1);
}
ShapeIntersection Triangle::GetIntersection(const Ray& ray, SurfacePoint s) const {
    V3 bary = v3(1 - (s.U + s.V), s.U, s.V);
    V3 p, n; V2 uv;
    TriBaryAttrs(*this, bary, &p, &n, &uv);
    ShapeIntersection r; r.P = p; r.UV = uv; r.T = s.T; r.Shading = Coordinate(n); r.Wr = -ray.D;
    return r;
}
bool Triangle::Intersect(const Ray& ray, SurfacePoint* sp) const {
    V3 edge1 = Pb() - Pa();
    V3 edge2 = Pc() - Pa();
    V3 pvec = Cross(ray.D, edge2);
    float det = Dot(edge1, pvec);
    if (Abs(det) < kFloatEpsilon) return false;
    float invDet = 1.0f / det;
    V3 tvec = ray.O - Pa();
    float u = Dot(tvec, pvec) * invDet;
    if (u < 0.0f || u > 1.0f) return false;
    V3 qvec = Cross(tvec, edge1);
    float v = Dot(ray.D, qvec) * invDet;
    if (v < 0.0f || u + v > 1.0f) return false;
    float t = Dot(edge2, qvec) * invDet;
    bool isInct = t >= ray.MinT && t <= ray.MaxT;
    if (isInct) { sp->U = u; sp->V = v; sp->T = t; }
    return isInct;
}
bool Triangle::IntersectP(const Ray& ray) const { SurfacePoint sp; return Intersect(ray, &sp); }
ShapeSurfacePoint Triangle::Sample(Rng& rand, float* pdf) const {
    V2 rng = rand.NextVec2();
    float alpha = 1 - Sqrt(1 - rng.x);
    float beta = rng.y * Sqrt(1 - rng.x);
    V3 bary = v3(alpha, beta, (1 - alpha - beta));
    V3 p, n; V2 uv;
    TriBaryAttrs(*this, bary, &p, &n, &uv);
    *pdf = 1.0f / Area;
    ShapeSurfacePoint r; r.P = p; r.UV = uv; r.Shading = Coordinate(n);
    return r;
}

/* ---- Sphere (Shapes/Sphere.cs) -------------------------------------------------- */
Sphere::Sphere(float r, V3 c, const M44& m2w, const M44& w2m) : Radius(r), Center(c), ModelToWorld(m2w), WorldToModel(w2m) {
    WorldBound = BBox(Center - v3s(Radius), Center + v3s(Radius));
}
/* System.Math.Min/Max(double, double): NaN-propagating, -0 < +0 */
static inline double netMinD(double a, double b) {
    if (a != b) { if (a == a) return a < b ? a : b; return a; }
    return std::signbit(a) ? a : b;
}
static inline double netMaxD(double a, double b) {
    if (a != b) { if (a == a) return b < a ? a : b; return a; }
    return std::signbit(b) ? a : b;
}
/* MathExt.SolveQuadratic (MathExt.cs:119-138) */
static inline bool SolveQuadratic(double a, double b, double c, double* x0o, double* x1o) {
    bool linearCase = a == 0.0;
    bool validLinear = linearCase && b != 0.0;
    double x0 = -c / b, x1 = -c / b;
    double discrim = b * b - 4.0 * a * c;
    bool validQuadratic = !linearCase && (discrim >= 0.0);
    if (validQuadratic) {
        double rootDiscrim = std::sqrt(discrim);
        double temp = -0.5 * (b + std::copysign(rootDiscrim, b));
        double x0p = temp / a;
        double x1p = c / temp;
        double x0m = netMinD(x0p, x1p), x1m = netMaxD(x0p, x1p);
        x0 = linearCase ? x0 : x0m;
        x1 = linearCase ? x0 : x1m;
    }
    *x0o = x0; *x1o = x1;
    return validLinear || validQuadratic;
}
static inline bool SphereSolve(const Sphere& s, const Ray& ray, double* nearT, double* farT) {
    double ox = (double)ray.O.x - (double)s.Center.x, oy = (double)ray.O.y - (double)s.Center.y, oz = (double)ray.O.z - (double)s.Center.z;
    double dx = ray.D.x, dy = ray.D.y, dz = ray.D.z;
    double a = (dx * dx + dy * dy) + dz * dz;
    double b = 2 * ((ox * dx + oy * dy) + oz * dz);
    double c = ((ox * ox + oy * oy) + oz * oz) - (double)Sqr(s.Radius);
    return SolveQuadratic(a, b, c, nearT, farT);
}
bool Sphere::IntersectP(const Ray& ray) const {
    double mint = ray.MinT, maxt = ray.MaxT, nearT, farT;
    bool found = SphereSolve(*this, ray, &nearT, &farT);
    bool outB = !(nearT <= maxt && farT >= mint);
    bool inB = nearT < mint && farT > maxt;
    return found && !outB && !inB;
}
bool Sphere::Intersect(const Ray& ray, SurfacePoint* sp) const {
    double mint = ray.MinT, maxt = ray.MaxT, nearT, farT;
    bool found = SphereSolve(*this, ray, &nearT, &farT);
    bool outB = !(nearT <= maxt && farT >= mint);
    bool inB = nearT < mint && farT > maxt;
    bool isHit = found && !outB && !inB;
    sp->U = 0; sp->V = 0; sp->T = nearT < mint ? (float)farT : (float)nearT;
    return isHit;
}
static inline V2 SphereUV(const Sphere& s, V3 n) {
    V3 local = TransformNormal(n, s.WorldToModel);
    float theta = Acos(-local.y);
    float phi = Atan2(-local.z, local.x) + kPI;
    return v2(phi / (2 * kPI), theta / kPI);
}
ShapeIntersection Sphere::GetIntersection(const Ray& ray, SurfacePoint s) const {
    float t = s.T;
    V3 n = Normalize(ray.At(t) - Center);
    V3 p = n * Radius + Center;
    ShapeIntersection r; r.P = p; r.UV = SphereUV(*this, n); r.T = t; r.Shading = Coordinate(n); r.Wr = -ray.D;
    return r;
}
ShapeSurfacePoint Sphere::Sample(Rng& rand, float* pdf) const {
    V3 rng = SquareToUniformSphere(rand.NextVec2());
    V3 n = Normalize(rng);
    ShapeSurfacePoint r; r.Shading = Coordinate(n); r.P = n * Radius + Center;
    *pdf = 1 / SurfaceArea();
    r.UV = SphereUV(*this, n);
    return r;
}

/* ---- Homogeneous medium + Henyey-Greenstein (Mediums/Homogeneous.cs, IPhaseFunction.cs) */
C3 Medium::Tr(const Ray& ray) const {
    float negLength = ray.MinT - ray.MaxT;
    C3 tr;
    tr.r = SigmaT.r == 0 ? 1.0f : Exp(SigmaT.r * negLength);
    tr.g = SigmaT.g == 0 ? 1.0f : Exp(SigmaT.g * negLength);
    tr.b = SigmaT.b == 0 ? 1.0f : Exp(SigmaT.b * negLength);
    return tr;
}
SampleMediumResult Medium::Sample(const Ray& ray, Rng& rand) const {
    int channel = rand.Next(3);
    C3 sigmaT = SigmaT;
    float samplingDensity = CGet(sigmaT, channel);
    float sampledDistance = -Log(1 - rand.NextFloat()) / samplingDensity;
    float distSurf = ray.MaxT - ray.MinT;
    SampleMediumResult r; r.M = this;
    if (sampledDistance < distSurf) {
        float t = ray.MinT + sampledDistance;
        V3 p = ray.At(t);
        C3 tr;
        tr.r = Exp(-sigmaT.r * sampledDistance);
        tr.g = Exp(-sigmaT.g * sampledDistance);
        tr.b = Exp(-sigmaT.b * sampledDistance);
        float pdf = (tr.r * sigmaT.r + tr.g * sigmaT.g + tr.b * sigmaT.b) / 3;
        if (pdf == 0) pdf = 0.0001f;
        r.P = p; r.Wo = -ray.D; r.Tr = tr * SigmaS / pdf; r.T = t; r.IsSampleMedium = true;
        return r;
    }
    C3 tr;
    tr.r = Exp(-SigmaT.r * distSurf);
    tr.g = Exp(-SigmaT.g * distSurf);
    tr.b = Exp(-SigmaT.b * distSurf);
    float pdf = (tr.r + tr.g + tr.b) / 3;
    if (pdf == 0) pdf = 0.0001f;
    r.Tr = tr / pdf; r.IsSampleMedium = false; r.P = v3s(0); r.Wo = v3s(0);
    return r;
}
static inline float HGValue(float cosTheta, float g) {
    float denom = 1 + g * g + 2 * g * cosTheta;
    return (1 / (4 * kPI)) * (1 - g * g) / (denom * Sqrt(denom));
}
static inline float HGClamp(float g) { return netClamp(g, -0.999f, 0.999f); }
float Medium::P(V3 wo, V3 wi) const { return HGValue(Dot(wo, wi), HGClamp(G)); }
SamplePhaseFunctionResult Medium::SampleWi(V3 wo, Rng& rand) const {
    float g = HGClamp(G);
    V2 rng = rand.NextVec2();
    float cosTheta;
    if (Abs(g) < 0.001f) cosTheta = 1 - 2 * rng.x;
    else {
        float sqrTerm = (1 - g * g) / (1 + g - 2 * g * rng.x);
        cosTheta = -(1 + g * g - sqrTerm * sqrTerm) / (2 * g);
    }
    float sinTheta = Sqrt(netMax(0, 1 - cosTheta * cosTheta));
    float phi = 2 * kPI * rng.y;
    Coordinate coord(wo);
    V3 wi = SphericalDirectionF(sinTheta, cosTheta, phi, coord.X, coord.Y, coord.Z);
    SamplePhaseFunctionResult r; r.P = HGValue(cosTheta, g); r.Wi = wi;
    return r;
}

/* ---- primitives (Primitive.cs) ------------------------------------------------------ */
bool GeometricPrimitive::IntersectP(const Ray& ray) const { return S->IntersectP(ray); }
bool GeometricPrimitive::Intersect(const Ray& ray, Intersection* inct) const {
    SurfacePoint sp;
    bool isHit = S->Intersect(ray, &sp);
    if (isHit) {
        ShapeIntersection s = S->GetIntersection(ray, sp);
        inct->P = s.P; inct->UV = s.UV; inct->T = s.T; inct->Shape = this; inct->Shading = s.Shading; inct->Wr = s.Wr;
        inct->prim_id = id; inct->sub_id = -1; inct->flags = 0; inct->bu = sp.U; inct->bv = sp.V;
    }
    return isHit;
}
bool ShapeWrapperPrimitive::IntersectP(const Ray& ray) const { return S->IntersectP(ray); }
bool ShapeWrapperPrimitive::Intersect(const Ray& ray, Intersection* inct) const {
    SurfacePoint sp;
    bool isHit = S->Intersect(ray, &sp);
    if (isHit) {
        ShapeIntersection s = S->GetIntersection(ray, sp);
        inct->P = s.P; inct->UV = s.UV; inct->T = s.T; inct->Shape = this; inct->Shading = s.Shading; inct->Wr = s.Wr;
        inct->prim_id = id; inct->sub_id = -1; inct->flags = 0; inct->bu = sp.U; inct->bv = sp.V;
    }
    return isHit;
}
InstancedPrimitive::InstancedPrimitive(const Primitive* inst, const M44& m2w, const M44& w2m, const Material* m, MediumAdapter med)
    : Instanced(inst), ModelToWorld(m2w), WorldToModel(w2m), Mat(m), Med(med) {
    Bound = BTransform(Instanced->WorldBound(), ModelToWorld);
}
bool InstancedPrimitive::IntersectP(const Ray& ray) const {
    cnt_inst();
    Ray modelRay = TransformRay(ray, WorldToModel);
    return Instanced->IntersectP(modelRay);
}
bool InstancedPrimitive::Intersect(const Ray& ray, Intersection* inct) const {
    cnt_inst();
    Ray modelRay = TransformRay(ray, WorldToModel);
    Intersection mi;
    bool anyHit = Instanced->Intersect(modelRay, &mi);
    if (anyHit) {
        V3 p = Transform(mi.P, ModelToWorld);
        V3 n = Normalize(TransformNormal(mi.N(), ModelToWorld));
        Coordinate coord(n);
        V3 wr = Normalize(TransformNormal(mi.Wr, ModelToWorld));
        inct->P = p; inct->UV = mi.UV; inct->T = Distance(ray.O, p); inct->Shape = this; inct->Shading = coord; inct->Wr = wr;
        inct->prim_id = id; inct->sub_id = mi.prim_id; inct->flags = mi.flags; inct->bu = mi.bu; inct->bv = mi.bv;
    }
    return anyHit;
}

/* ---- Bvh (Accelerators/Bvh.cs) ------------------------------------------------------- */
struct BVHPrimitiveInfo { int PrimitiveNumber; BBox Bounds; V3 Centroid; };
struct BVHBuildNode {
    BBox Bounds; BVHBuildNode* Left = nullptr; BVHBuildNode* Right = nullptr;
    int SplitAxis = 0, FirstPrimIndex = 0, PrimitiveCount = 0;
};
/* MathExt.Partition (MathExt.cs:170-201), called with `end - 1` as last */
template <class F>
static int Partition(std::vector<BVHPrimitiveInfo>& list, int begin, int end, F func) {
    int first = begin, last = end;
    while (true) {
        while (true) {
            if (first == last) return first;
            if (!func(list[first])) break;
            ++first;
        }
        while (!func(list[last])) {
            if (first == last) return first;
            last--;
        }
        std::swap(list[first], list[last]);
        first++;
    }
}
struct BvhBuilder {
    const std::vector<const Primitive*>& prims;
    std::vector<const Primitive*>& ordered;
    std::vector<std::unique_ptr<BVHBuildNode>> store;
    int maxPrims; int totalNodes = 0; int leafCount = 0;
    BvhBuilder(const std::vector<const Primitive*>& p, std::vector<const Primitive*>& o, int mp) : prims(p), ordered(o), maxPrims(mp) {}
    BVHBuildNode* MakeLeaf(std::vector<BVHPrimitiveInfo>& info, int start, int end, const BBox& bounds) {
        int first = (int)ordered.size();
        for (int i = start; i < end; i++) ordered.push_back(prims[info[i].PrimitiveNumber]);
        store.emplace_back(new BVHBuildNode());
        BVHBuildNode* n = store.back().get();
        n->FirstPrimIndex = first; n->PrimitiveCount = end - start; n->Bounds = bounds;
        leafCount++;
        return n;
    }
    BVHBuildNode* Build(std::vector<BVHPrimitiveInfo>& info, int start, int end) {
        totalNodes++;
        BBox bounds;
        for (int i = start; i < end; i++) bounds.Union(info[i].Bounds);
        int nPrimitives = end - start;
        if (nPrimitives == 1) return MakeLeaf(info, start, end, bounds);
        BBox centroidBounds;
        for (int i = start; i < end; i++) centroidBounds.ExpendBy(info[i].Centroid);
        int dim = centroidBounds.MaximumExtent();
        int mid = (start + end) / 2;
        if (Get(centroidBounds.Max, dim) == Get(centroidBounds.Min, dim)) return MakeLeaf(info, start, end, bounds);
        if (nPrimitives <= 2) {
            mid = (start + end) / 2;
            /* List.Sort of two elements: SwapIfGreater */
            float lv = Get(info[start].Centroid, dim), rv = Get(info[start + 1].Centroid, dim);
            int cmp = (lv == rv) ? 0 : (lv < rv ? -1 : 1);
            if (cmp > 0) std::swap(info[start], info[start + 1]);
        } else {
            const int nBuckets = 12;
            int count[nBuckets]; BBox bb[nBuckets];
            for (int i = 0; i < nBuckets; i++) { count[i] = 0; bb[i] = BBox(); }
            for (int i = start; i < end; i++) {
                V3 off = centroidBounds.Offset(info[i].Centroid);
                int b = netF2I((float)nBuckets * Get(off, dim));
                if (b == nBuckets) b = nBuckets - 1;
                count[b]++;
                bb[b].Union(info[i].Bounds);
            }
            float cost[nBuckets - 1];
            for (int i = 0; i < nBuckets - 1; i++) {
                BBox b0, b1; int count0 = 0, count1 = 0;
                for (int j = 0; j <= i; j++) { b0.Union(bb[j]); count0 += count[j]; }
                for (int j = i + 1; j < nBuckets; j++) { b1.Union(bb[j]); count1 += count[j]; }
                cost[i] = 1 + ((float)count0 * b0.SurfaceArea() + (float)count1 * b1.SurfaceArea()) / bounds.SurfaceArea();
            }
            float minCost = cost[0]; int minB = 0;
            for (int i = 1; i < nBuckets - 1; i++) if (cost[i] < minCost) { minCost = cost[i]; minB = i; }
            float leafCost = (float)nPrimitives;
            if (nPrimitives > maxPrims || minCost < leafCost) {
                mid = Partition(info, start, end - 1, [&](const BVHPrimitiveInfo& pi) {
                    V3 off = centroidBounds.Offset(pi.Centroid);
                    int b = netF2I((float)nBuckets * Get(off, dim));
                    return b <= minB;
                });
            } else {
                return MakeLeaf(info, start, end, bounds);
            }
        }
        BVHBuildNode* l = Build(info, start, mid);
        BVHBuildNode* r = Build(info, mid, end);
        store.emplace_back(new BVHBuildNode());
        BVHBuildNode* n = store.back().get();
        n->Left = l; n->Right = r; n->Bounds = BUnion(l->Bounds, r->Bounds); n->SplitAxis = dim; n->PrimitiveCount = 0;
        return n;
    }
};
static int Flatten(std::vector<LinearBVHNode>& nodes, const BVHBuildNode* node, int* offset) {
    LinearBVHNode& ln = nodes[*offset];
    ln.Bounds = node->Bounds;
    int my = (*offset)++;
    if (node->PrimitiveCount > 0) {
        nodes[my].PrimitivesIndex = node->FirstPrimIndex;
        nodes[my].PrimitiveCount = (uint16_t)node->PrimitiveCount;
        nodes[my].Axis = 0;
    } else {
        nodes[my].Axis = (uint8_t)node->SplitAxis;
        nodes[my].PrimitiveCount = 0;
        Flatten(nodes, node->Left, offset);
        int second = Flatten(nodes, node->Right, offset);
        nodes[my].PrimitivesIndex = second;
    }
    return my;
}
Bvh::Bvh(const std::vector<const Primitive*>& p, int maxPrimsInNode) : maxPrims(maxPrimsInNode) {
    if (p.empty()) return;
    std::vector<BVHPrimitiveInfo> info(p.size());
    for (size_t i = 0; i < p.size(); i++) {
        BBox b = p[i]->WorldBound();
        info[i].PrimitiveNumber = (int)i; info[i].Bounds = b;
        info[i].Centroid = 0.5f * b.Min + 0.5f * b.Max;
    }
    BvhBuilder builder(p, prims, maxPrims);
    prims.reserve(p.size());
    BVHBuildNode* root = builder.Build(info, 0, (int)p.size());
    leafCount = builder.leafCount;
    nodes.resize(builder.totalNodes);
    int offset = 0;
    Flatten(nodes, root, &offset);
}
/* thread-local flag raised when the 64-entry traversal stack overflows
 * (the reference throws IndexOutOfRangeException there). */
thread_local bool tl_stack_overflow = false;
bool Bvh::IntersectP(const Ray& ray) const {
    if (nodes.empty()) return false;
    bool dirIsNeg[3] = {ray.InvD.x < 0, ray.InvD.y < 0, ray.InvD.z < 0};
    int nodesToVisit[64];
    int toVisitOffset = 0, cur = 0;
    while (true) {
        const LinearBVHNode& node = nodes[cur];
        cnt_node();
        if (node.Bounds.Intersect(ray)) {
            if (node.PrimitiveCount > 0) {
                for (int i = 0; i < node.PrimitiveCount; ++i) {
                    cnt_prim();
                    if (prims[node.PrimitivesIndex + i]->IntersectP(ray)) return true;
                }
                if (toVisitOffset == 0) break;
                cur = nodesToVisit[--toVisitOffset];
            } else {
                if (toVisitOffset == 64) { tl_stack_overflow = true; return false; }
                if (dirIsNeg[node.Axis]) { nodesToVisit[toVisitOffset++] = cur + 1; cur = node.PrimitivesIndex; }
                else { nodesToVisit[toVisitOffset++] = node.PrimitivesIndex; cur = cur + 1; }
            }
        } else {
            if (toVisitOffset == 0) break;
            cur = nodesToVisit[--toVisitOffset];
        }
    }
    return false;
}
bool Bvh::Intersect(const Ray& rayIn, Intersection* inct) const {
    if (nodes.empty()) return false;
    Ray ray = rayIn;
    bool dirIsNeg[3] = {ray.InvD.x < 0, ray.InvD.y < 0, ray.InvD.z < 0};
    int nodesToVisit[64];
    int toVisitOffset = 0, cur = 0;
    Intersection now; now.T = kFloatMax;
    bool anyHit = false; uint32_t flags = 0;
    while (true) {
        const LinearBVHNode& node = nodes[cur];
        cnt_node();
        if (node.Bounds.Intersect(ray)) {
            if (node.PrimitiveCount > 0) {
                for (int i = 0; i < node.PrimitiveCount; ++i) {
                    Intersection th;
                    cnt_prim();
                    if (prims[node.PrimitivesIndex + i]->Intersect(ray, &th)) {
                        anyHit = true;
                        flags |= th.flags;
                        if (th.T < now.T) { now = th; ray.MaxT = th.T; }
                        else if (th.T == now.T) flags |= RT_HIT_TIE;
                    }
                }
                if (toVisitOffset == 0) break;
                cur = nodesToVisit[--toVisitOffset];
            } else {
                if (toVisitOffset == 64) { tl_stack_overflow = true; break; }
                if (dirIsNeg[node.Axis]) { nodesToVisit[toVisitOffset++] = cur + 1; cur = node.PrimitivesIndex; }
                else { nodesToVisit[toVisitOffset++] = node.PrimitivesIndex; cur = cur + 1; }
            }
        } else {
            if (toVisitOffset == 0) break;
            cur = nodesToVisit[--toVisitOffset];
        }
    }
    if (anyHit) { *inct = now; inct->flags = flags; }
    return anyHit;
}

/* ---- microfacet distributions (Bxdf/Microfacet.cs) ------------------------------------ */
struct Dist {
    int type; float ax, ay;
    Dist(int t, float roughness, float anisotropic) : type(t) {
        float k = anisotropic;
        ax = netMax(roughness * roughness * (1 + k), 0.001f);
        ay = netMax(roughness * roughness * (1 - k), 0.001f);
    }
    float D(V3 wh) const {
        float tan2Theta = Tan2Theta(wh);
        if (isinf_(tan2Theta)) return 0.0f;
        float cos4Theta = Cos2Theta(wh) * Cos2Theta(wh);
        if (type == RT_DIST_BECKMANN)
            return Exp(-tan2Theta * (Cos2Phi(wh) / (ax * ax) + Sin2Phi(wh) / (ay * ay))) / (kPI * ax * ay * cos4Theta);
        float e = (Cos2Phi(wh) / (ax * ax) + Sin2Phi(wh) / (ay * ay)) * tan2Theta;
        return 1 / (kPI * ax * ay * cos4Theta * (1 + e) * (1 + e));
    }
    float Lambda(V3 w) const {
        float absTanTheta = Abs(TanTheta(w));
        if (isinf_(absTanTheta)) return 0.0f;
        float alpha = Sqrt(Cos2Phi(w) * ax * ax + Sin2Phi(w) * ay * ay);
        if (type == RT_DIST_BECKMANN) {
            float a = 1 / (alpha * absTanTheta);
            if (a >= 1.6f) return 0;
            return (1 - 1.259f * a + 0.396f * a * a) / (3.535f * a + 2.181f * a * a);
        }
        float alpha2Tan2Theta = (alpha * absTanTheta) * (alpha * absTanTheta);
        return (-1 + Sqrt(1.0f + alpha2Tan2Theta)) / 2;
    }
    float G(V3 wo, V3 wi) const { return 1 / (1 + Lambda(wo) + Lambda(wi)); }
    float Pdf(V3 /*wo*/, V3 wh) const { return D(wh) * AbsCosTheta(wh); }
    V3 SampleWh(V3 wo, Rng& rand) const {
        if (type == RT_DIST_BECKMANN) {
            float tan2Theta, phi;
            V2 u = rand.NextVec2();
            if (ax == ay) {
                float logSample = Log(1 - u.x);
                tan2Theta = -ax * ax * logSample;
                phi = u.y * 2 * kPI;
            } else {
                float logSample = Log(1 - u.x);
                phi = Atan(ay / ax * Tan(2 * kPI * u.y + 0.5f * kPI));
                if (u.y > 0.5f) phi += kPI;
                float sinPhi = Sin(phi), cosPhi = Cos(phi);
                float ax2 = ax * ax, ay2 = ay * ay;
                tan2Theta = -logSample / (cosPhi * cosPhi / ax2 + sinPhi * sinPhi / ay2);
            }
            float cosTheta = 1 / Sqrt(1 + tan2Theta);
            float sinTheta = Sqrt(netMax(0, 1 - cosTheta * cosTheta));
            V3 wh = SphericalDirection(sinTheta, cosTheta, phi);
            if (!SameHemisphere(wo, wh)) wh = -wh;
            return wh;
        }
        /* SampleWhGGX */
        V2 u = rand.NextVec2();
        float phi = (2 * kPI) * u.y;
        float cosTheta;
        if (ax == ay) {
            float tanTheta2 = ax * ax * u.x / (1.0f - u.x);
            cosTheta = 1 / Sqrt(1 + tanTheta2);
        } else {
            phi = Atan(ay / ax * Tan(2 * kPI * u.y + .5f * kPI));
            if (u.y > 0.5f) phi += kPI;
            float sinPhi = Sin(phi), cosPhi = Cos(phi);
            float ax2 = ax * ax, ay2 = ay * ay;
            float alpha2 = 1 / (cosPhi * cosPhi / ax2 + sinPhi * sinPhi / ay2);
            float tanTheta2 = alpha2 * u.x / (1 - u.x);
            cosTheta = 1 / Sqrt(1 + tanTheta2);
        }
        float sinTheta = Sqrt(netMax(0.0f, 1.0f - cosTheta * cosTheta));
        V3 wh = SphericalDirection(sinTheta, cosTheta, phi);
        if (!SameHemisphere(wo, wh)) wh = -wh;
        return wh;
    }
};

/* ---- Fresnel (Bxdf/Fresnel.cs:50-95) --------------------------------------------------- */
static float DielectricFunc(float cosThetaI, float etaI, float etaT) {
    cosThetaI = netClamp(cosThetaI, -1, 1);
    bool entering = cosThetaI > 0.0f;
    if (!entering) { float t = etaI; etaI = etaT; etaT = t; cosThetaI = Abs(cosThetaI); }
    float sinThetaI = Sqrt(netMax(0, 1 - cosThetaI * cosThetaI));
    float sinThetaT = etaI / etaT * sinThetaI;
    if (sinThetaT >= 1) return 1;
    float cosThetaT = Sqrt(netMax(0, 1 - sinThetaT * sinThetaT));
    float rparl = ((etaT * cosThetaI) - (etaI * cosThetaT)) / ((etaT * cosThetaI) + (etaI * cosThetaT));
    float rperp = ((etaI * cosThetaI) - (etaT * cosThetaT)) / ((etaI * cosThetaI) + (etaT * cosThetaT));
    return (rparl * rparl + rperp * rperp) / 2;
}
static C3 ConductorFunc(float cosThetaI, C3 etai, C3 etat, C3 k) {
    cosThetaI = netClamp(cosThetaI, -1, 1);
    C3 eta = etat / etai;
    C3 etak = k / etai;
    float cosThetaI2 = cosThetaI * cosThetaI;
    float sinThetaI2 = 1.0f - cosThetaI2;
    C3 eta2 = eta * eta;
    C3 etak2 = etak * etak;
    C3 t0 = eta2 - etak2 - sinThetaI2;
    C3 s = t0 * t0 + 4 * eta2 * etak2;
    C3 a2plusb2 = c3(Sqrt(s.r), Sqrt(s.g), Sqrt(s.b));
    C3 t1 = a2plusb2 + cosThetaI2;
    C3 s2 = 0.5f * (a2plusb2 + t0);
    C3 a = c3(Sqrt(s2.r), Sqrt(s2.g), Sqrt(s2.b));
    C3 t2 = 2 * cosThetaI * a;
    C3 Rs = (t1 - t2) / (t1 + t2);
    C3 t3 = cosThetaI2 * a2plusb2 + sinThetaI2 * sinThetaI2;
    C3 t4 = t2 * sinThetaI2;
    C3 Rp = Rs * (t3 - t4) / (t3 + t4);
    return 0.5f * (Rp + Rs);
}
/* MicrofacetReflectionBrdf<TFresnel, TMicrofacet> (Bxdf/MicrofacetReflectionBrdf.cs) with
 * fresnel = conductor (fr_kind 0) or dielectric (fr_kind 1) */
struct MicroRefl {
    C3 R; int frKind; C3 etaT, k; float dEtaI, dEtaT; const Dist& D;
    C3 Fresnel(float cosI) const {
        if (frKind == 0) return ConductorFunc(cosI, c3s(1.0f), etaT, k);
        return c3s(DielectricFunc(cosI, dEtaI, dEtaT));
    }
    C3 Fr(V3 wo, V3 wi) const {
        if (!SameHemisphere(wo, wi)) return c3s(0.0f);
        float cosThetaO = AbsCosTheta(wo), cosThetaI = AbsCosTheta(wi);
        V3 wh = wi + wo;
        if (cosThetaI == 0 || cosThetaO == 0) return c3s(0);
        if (wh.x == 0 && wh.y == 0 && wh.z == 0) return c3s(0);
        wh = Normalize(wh);
        C3 f = Fresnel(Dot(wi, Faceforward(wh, v3(0, 0, 1))));
        float d = D.D(wh);
        float g = D.G(wo, wi);
        return R * CAbs((d * g * f) / (4 * cosThetaI * cosThetaO));
    }
    float Pdf(V3 wo, V3 wi) const {
        if (!SameHemisphere(wo, wi)) return 0;
        V3 wh = Normalize(wo + wi);
        return D.Pdf(wo, wh) / (4 * Dot(wo, wh));
    }
    SampleBxdfResult Sample(V3 wo, Rng& rand) const {
        SampleBxdfResult r;
        if (CosTheta(wo) == 0) return r;
        V3 wh = D.SampleWh(wo, rand);
        if (Dot(wo, wh) < 0) return r;
        V3 wi = Reflect(-wo, wh);
        if (!SameHemisphere(wo, wi)) return r;
        r.Pdf = D.Pdf(wo, wh) / (4 * Dot(wi, wh));
        r.Fr = Fr(wo, wi);
        r.Wi = wi; r.Type = Reflection | Glossy;
        return r;
    }
};
/* LambertianReflectionBrdf (Bxdf/LambertianReflectionBrdf.cs) */
static inline C3 LambFr(C3 R, V3 wo, V3 wi) { return SameHemisphere(wo, wi) ? R / kPI : c3s(0); }
static inline float LambPdf(V3 wo, V3 wi) { return SameHemisphere(wo, wi) ? AbsCosTheta(wi) / kPI : 0.0f; }
static inline SampleBxdfResult LambSample(C3 R, V3 wo, Rng& rand) {
    SampleBxdfResult r;
    V3 wi = Normalize(SquareToCosineHemisphere(rand.NextVec2()));
    if (wo.z < 0) wi.z *= -1;
    if (!SameHemisphere(wo, wi)) return r;
    r.Pdf = LambPdf(wo, wi); r.Fr = R / kPI; r.Wi = wi; r.Type = Reflection | Diffuse_;
    return r;
}

/* ---- materials ------------------------------------------------------------------------ */
/* `importance`: TransportMode.Importance (Material.cs:6-10) drops the 1/eta^2
 * radiance scaling of refraction (RoughGlass.cs:63,161, FresnelSpecularBsdf.cs:58) */
static C3 GlassFr(const Material& m, V3 wo, V3 wi, V2 uv, const Dist& dist, bool importance) { /* RoughGlass.FrImpl */
    C3 r = m.R->Sample(uv), t = m.T->Sample(uv);
    bool isReflect = SameHemisphere(wo, wi);
    bool entering = CosTheta(wo) > 0;
    float etaI = entering ? m.etaA : m.etaB;
    float etaT = entering ? m.etaB : m.etaA;
    float eta = isReflect ? 1 : etaT / etaI;
    V3 wh = Normalize(wo + wi * eta);
    if (CosTheta(wh) < 0) wh = -wh;
    float sqrtDenom = Dot(wo, wh) + eta * Dot(wi, wh);
    float d = dist.D(wh);
    float g = dist.G(wo, wi);
    float f = DielectricFunc(Dot(wo, wh), etaI, etaT);
    C3 bsdf;
    if (isReflect) {
        bsdf = r * (d * g * f / (4.0f * CosTheta(wi) * CosTheta(wo)));
    } else {
        if (Dot(wo, wh) * Dot(wi, wh) > 0) return c3s(0);
        float factor = importance ? 1.0f : 1 / eta;
        bsdf = (1 - f) * t * Abs(d * g * eta * eta * AbsDot(wi, wh) * AbsDot(wo, wh) * factor * factor /
                                  (CosTheta(wo) * CosTheta(wi) * sqrtDenom * sqrtDenom));
    }
    return IsValid(bsdf) ? bsdf : c3s(0.0f);
}
static float GlassPdf(const Material& m, V3 wo, V3 wi, const Dist& dist) { /* RoughGlass.PdfImpl */
    bool isReflect = SameHemisphere(wo, wi);
    bool entering = CosTheta(wo) > 0;
    float etaI = entering ? m.etaA : m.etaB;
    float etaT = entering ? m.etaB : m.etaA;
    float pdf;
    if (isReflect) {
        V3 wh = Normalize(wo + wi);
        if (CosTheta(wh) < 0) wh = -wh;
        if (Dot(wo, wh) * CosTheta(wo) <= 0 || Dot(wi, wh) * CosTheta(wi) <= 0) return 0.0f;
        float jacobian = 1.0f / (4.0f * AbsDot(wh, wi));
        float f = DielectricFunc(Dot(wo, wh), etaI, etaT);
        pdf = dist.Pdf(wo, wh) * jacobian * f;
    } else {
        float eta = etaT / etaI;
        V3 wh = Normalize(wo + wi * eta);
        if (CosTheta(wh) < 0) wh = -wh;
        if (Dot(wo, wh) * Dot(wi, wh) > 0) return 0.0f;
        if (Dot(wo, wh) * CosTheta(wo) <= 0 || Dot(wi, wh) * CosTheta(wi) <= 0) return 0.0f;
        float sqrtDenom = Dot(wo, wh) + eta * Dot(wi, wh);
        float dwhdwi = Abs((eta * eta * Dot(wi, wh)) / (sqrtDenom * sqrtDenom));
        float f = DielectricFunc(Dot(wo, wh), etaI, etaT);
        pdf = dist.Pdf(wo, wh) * dwhdwi * (1 - f);
    }
    return (isinf_(pdf) || isnan_(pdf)) ? 0.0f : pdf;
}
static SampleBxdfResult GlassSample(const Material& m, V3 wo, V2 uv, Rng& rand, const Dist& dist, bool importance) { /* RoughGlass.SampleImpl */
    SampleBxdfResult res;
    C3 r = m.R->Sample(uv), t = m.T->Sample(uv);
    V3 wh = dist.SampleWh(wo, rand);
    float f = DielectricFunc(Dot(wo, wh), m.etaA, m.etaB);
    if (rand.NextFloat() < f) {
        V3 wi = Reflect(-wo, wh);
        if (!SameHemisphere(wo, wi)) return res;
        float d = dist.D(wh);
        float g = dist.G(wo, wi);
        C3 brdf = r * (d * g * f / (4.0f * CosTheta(wi) * CosTheta(wo)));
        float jacobian = 1.0f / (4.0f * AbsDot(wh, wi));
        float pdf = dist.Pdf(wo, wh) * jacobian * f;
        if (isinf_(pdf) || isnan_(pdf) || !IsValid(brdf)) return res;
        res.Wi = wi; res.Fr = brdf; res.Pdf = pdf; res.Type = Reflection | Glossy;
        return res;
    }
    bool entering = CosTheta(wo) > 0;
    float etaI = entering ? m.etaA : m.etaB;
    float etaT = entering ? m.etaB : m.etaA;
    float eta = etaT / etaI;
    V3 wi;
    if (Refract(wo, wh, etaI / etaT, &wi)) {
        if (Dot(wo, wh) * Dot(wi, wh) > 0) return res;
    } else {
        wi = Reflect(-wo, wh);
        eta = 1;
    }
    float sqrtDenom = Dot(wo, wh) + eta * Dot(wi, wh);
    float factor = importance ? 1.0f : 1 / eta;
    float d = dist.D(wh);
    float g = dist.G(wo, wi);
    C3 btdf = (1 - f) * t * Abs(d * g * eta * eta * AbsDot(wi, wh) * AbsDot(wo, wh) * factor * factor /
                                 (CosTheta(wo) * CosTheta(wi) * sqrtDenom * sqrtDenom));
    float dwhdwi = Abs((eta * eta * Dot(wi, wh)) / (sqrtDenom * sqrtDenom));
    float pdf = dist.Pdf(wo, wh) * dwhdwi * (1 - f);
    if (isinf_(pdf) || isnan_(pdf) || !IsValid(btdf)) return res;
    res.Wi = wi; res.Fr = btdf; res.Pdf = pdf; res.Type = Transmission | Glossy;
    return res;
}
static inline bool OneSidedReject(const Material& m, V3 wo, V3 wi) {
    return (CosTheta(wo) <= 0 || CosTheta(wi) <= 0) && !m.twoSided;
}
static C3 PlasticFr(const Material& m, V3 wo, V3 wi, const Dist& dist, C3 r) { /* RoughPlastic.FrImpl */
    if (OneSidedReject(m, wo, wi)) return c3s(0.0f);
    C3 diffuse = LambFr(r, wo, wi);
    MicroRefl mr{r, 1, c3s(0), c3s(0), m.etaA, m.etaB, dist};
    C3 glossy = mr.Fr(wo, wi);
    return m.kd * diffuse + m.ks * glossy;
}
static float PlasticPdf(const Material& m, V3 wo, V3 wi, const Dist& dist, C3 r) { /* RoughPlastic.PdfImpl */
    if (OneSidedReject(m, wo, wi)) return 0.0f;
    float p = m.ks / (m.kd + m.ks);
    float diffuse = LambPdf(wo, wi);
    MicroRefl mr{r, 1, c3s(0), c3s(0), m.etaA, m.etaB, dist};
    float glossy = mr.Pdf(wo, wi);
    return (1 - p) * diffuse + p * glossy;
}

C3 Material::Fr(V3 wo, V3 wi, const Intersection& inct, bool importance) const {
    switch (type) {
    case RT_MAT_DIFFUSE:
        if (OneSidedReject(*this, wo, wi)) return c3s(0.0f);
        return LambFr(R->Sample(inct.UV), wo, wi);
    case RT_MAT_ROUGH_METAL: {
        Dist d(dist, Rough->Sample(inct.UV).r, Anis->Sample(inct.UV).r);
        if (OneSidedReject(*this, wo, wi)) return c3s(0.0f);
        MicroRefl mr{c3s(1.0f), 0, Eta, K, 0, 0, d};
        return mr.Fr(wo, wi);
    }
    case RT_MAT_ROUGH_GLASS: {
        Dist d(dist, Rough->Sample(inct.UV).r, Anis->Sample(inct.UV).r);
        return GlassFr(*this, wo, wi, inct.UV, d, importance);
    }
    case RT_MAT_ROUGH_PLASTIC: {
        Dist d(dist, Rough->Sample(inct.UV).r, Anis->Sample(inct.UV).r);
        return PlasticFr(*this, wo, wi, d, R->Sample(inct.UV));
    }
    default: /* perfect mirror / glass: delta lobes evaluate to black */
        return c3s(0.0f);
    }
}
float Material::Pdf(V3 wo, V3 wi, const Intersection& inct) const {
    switch (type) {
    case RT_MAT_DIFFUSE:
        if (OneSidedReject(*this, wo, wi)) return 0.0f;
        return LambPdf(wo, wi);
    case RT_MAT_ROUGH_METAL: {
        Dist d(dist, Rough->Sample(inct.UV).r, Anis->Sample(inct.UV).r);
        if (OneSidedReject(*this, wo, wi)) return 0.0f;
        MicroRefl mr{c3s(1.0f), 0, Eta, K, 0, 0, d};
        return mr.Pdf(wo, wi);
    }
    case RT_MAT_ROUGH_GLASS: {
        Dist d(dist, Rough->Sample(inct.UV).r, Anis->Sample(inct.UV).r);
        return GlassPdf(*this, wo, wi, d);
    }
    case RT_MAT_ROUGH_PLASTIC: {
        Dist d(dist, Rough->Sample(inct.UV).r, Anis->Sample(inct.UV).r);
        return PlasticPdf(*this, wo, wi, d, R->Sample(inct.UV));
    }
    default:
        return 0.0f;
    }
}
SampleBxdfResult Material::Sample(V3 wo, const Intersection& inct, Rng& rand, bool importance) const {
    SampleBxdfResult res;
    switch (type) {
    case RT_MAT_DIFFUSE:
        if (CosTheta(wo) <= 0 && !twoSided) return res;
        return LambSample(R->Sample(inct.UV), wo, rand);
    case RT_MAT_ROUGH_METAL: {
        Dist d(dist, Rough->Sample(inct.UV).r, Anis->Sample(inct.UV).r);
        if (CosTheta(wo) <= 0 && !twoSided) return res;
        MicroRefl mr{c3s(1.0f), 0, Eta, K, 0, 0, d};
        return mr.Sample(wo, rand);
    }
    case RT_MAT_ROUGH_GLASS: {
        Dist d(dist, Rough->Sample(inct.UV).r, Anis->Sample(inct.UV).r);
        return GlassSample(*this, wo, inct.UV, rand, d, importance);
    }
    case RT_MAT_ROUGH_PLASTIC: {
        Dist d(dist, Rough->Sample(inct.UV).r, Anis->Sample(inct.UV).r);
        if (CosTheta(wo) <= 0 && !twoSided) return res;
        C3 r = R->Sample(inct.UV);
        float p = ks / (kd + ks);
        MicroRefl mr{r, 1, c3s(0), c3s(0), etaA, etaB, d};
        SampleBxdfResult glossy = mr.Sample(wo, rand);
        SampleBxdfResult diffuse = LambSample(r, wo, rand);
        V3 wi; int tp;
        if (rand.NextFloat() < p) { wi = glossy.Wi; tp = glossy.Type; }
        else { wi = diffuse.Wi; tp = diffuse.Type; }
        res.Pdf = PlasticPdf(*this, wo, wi, d, r);
        res.Fr = PlasticFr(*this, wo, wi, d, r);
        res.Wi = wi; res.Type = tp;
        return res;
    }
    case RT_MAT_PERFECT_MIRROR: { /* PerfectMirror + SpecularReflectionBrdf */
        if (CosTheta(wo) <= 0 && !twoSided) return res;
        C3 R_ = R->Sample(inct.UV);
        if (AbsCosTheta(wo) == 0) return res;
        V3 wi = v3(-wo.x, -wo.y, wo.z);
        res.Wi = wi; res.Fr = R_ / AbsCosTheta(wi); res.Pdf = 1.0f; res.Type = Reflection | Specular;
        return res;
    }
    case RT_MAT_PERFECT_GLASS: { /* PerfectGlass + FresnelSpecularBsdf */
        C3 R_ = R->Sample(inct.UV), T_ = T->Sample(inct.UV);
        float f = DielectricFunc(CosTheta(wo), etaA, etaB);
        if (rand.NextFloat() < f) {
            if (CosTheta(wo) == 0) return res;
            V3 wi = v3(-wo.x, -wo.y, wo.z);
            res.Wi = wi; res.Fr = f * R_ / AbsCosTheta(wi); res.Pdf = f; res.Type = Reflection | Specular;
            return res;
        }
        bool entering = CosTheta(wo) > 0;
        float etaI = entering ? etaA : etaB;
        float etaT = entering ? etaB : etaA;
        V3 n = entering ? v3(0, 0, 1) : v3(0, 0, -1);
        V3 wi;
        if (!Refract(wo, n, etaI / etaT, &wi) || CosTheta(wi) == 0.0f) return res;
        C3 ft = T_ * (1.0f - f);
        if (!importance) ft = ft * ((etaI * etaI) / (etaT * etaT));
        ft = ft / AbsCosTheta(wi);
        res.Wi = wi; res.Fr = ft; res.Pdf = 1 - f; res.Type = Transmission | Specular;
        return res;
    }
    }
    return res;
}

/* ---- lights ------------------------------------------------------------------------------- */
float AreaLight::PdfLi(LightEvalParam inct, V3 wi) const { /* DiffuseAreaLight.cs:31-46 */
    Ray ray(inct.P, wi);
    SurfacePoint point;
    if (!S->Intersect(ray, &point)) return 0.0f;
    ShapeIntersection hit = S->GetIntersection(ray, point);
    float pdf = LengthSquared(inct.P - hit.P) / (AbsDot(hit.Shading.Z, -wi) * S->SurfaceArea());
    if (isinf_(pdf)) pdf = 0.0f;
    return pdf;
}
SampleLightResult AreaLight::SampleLi(LightEvalParam inct, Rng& rand) const { /* DiffuseAreaLight.cs:48-68 */
    float shapePdf;
    ShapeSurfacePoint shape = S->Sample(rand, &shapePdf);
    V3 wi = shape.P - inct.P;
    C3 li = (Dot(shape.Shading.Z, -wi) > 0) ? LightEmit : c3s(0.0f);
    float pdf;
    if (LengthSquared(wi) == 0) pdf = 0.0f;
    else {
        wi = Normalize(wi);
        pdf = shapePdf * LengthSquared(inct.P - shape.P) / AbsDot(shape.Shading.Z, -wi);
        if (isinf_(pdf)) pdf = 0.0f;
    }
    SampleLightResult r; r.P = shape.P; r.Li = li; r.Wi = wi; r.Pdf = pdf;
    return r;
}
Distribution1D::Distribution1D(const float* p, int n) { /* Distribution1D.cs:19-49 */
    pdf.assign(p, p + n);
    cdf.assign(n + 1, 0.0f);
    cdf[0] = 0;
    for (int i = 1; i < n + 1; ++i) cdf[i] = cdf[i - 1] + pdf[i - 1] / (float)n;
    integration = cdf[n];
    if (integration == 0) { for (int i = 1; i < n + 1; i++) cdf[i] = (float)i / (float)n; }
    else { for (int i = 1; i < n + 1; i++) cdf[i] /= integration; }
}
int Distribution1D::FindInterval(float u) const { /* Distribution1D.cs:51-69 */
    int first = 0, len = (int)cdf.size();
    while (len > 0) {
        int half = len >> 1, middle = first + half;
        if (cdf[middle] <= u) { first = middle + 1; len -= half + 1; }
        else len = half;
    }
    return netClampI(first - 1, 0, (int)cdf.size() - 2);
}
float Distribution1D::SampleContinuous(float u, float* pdfOut, int* offset) const {
    *offset = FindInterval(u);
    float du = u - cdf[*offset];
    if ((cdf[*offset + 1] - cdf[*offset]) > 0) du /= cdf[*offset + 1] - cdf[*offset];
    *pdfOut = ContinuousPdf(*offset);
    return ((float)*offset + du) / (float)Count();
}
Distribution2D::Distribution2D(const float* data, int nu, int nv) { /* Distribution2D.cs:14-30 */
    conditional.reserve(nv);
    for (int v = 0; v < nv; v++) conditional.emplace_back(data + (size_t)v * nu, nu);
    std::vector<float> marg(nv);
    for (int v = 0; v < nv; v++) marg[v] = conditional[v].integration;
    marginal = Distribution1D(marg.data(), nv);
}
V2 Distribution2D::SampleContinuous(V2 u, float* pdf, int* offV, int* offU) const {
    float pdf1, pdf0; int vj, vi;
    float d1 = marginal.SampleContinuous(u.y, &pdf1, &vj);
    float d0 = conditional[vj].SampleContinuous(u.x, &pdf0, &vi);
    *pdf = pdf0 * pdf1;
    *offV = vj; *offU = vi;
    return v2(d0, d1);
}
float Distribution2D::ContinuousPdf(float u, float v) const {
    int nu = conditional[0].Count(), nv = marginal.Count();
    int iu = netClampI(netF2I(u * (float)nu), 0, nu - 1);
    int iv = netClampI(netF2I(v * (float)nv), 0, nv - 1);
    return conditional[iv].pdf[iu] / marginal.integration;
}
InfiniteAreaLight::InfiniteAreaLight(const M44& m2w, const M44& w2m, const Texture2D* map)
    : ModelToWorld(m2w), WorldToModel(w2m), Map(map) { /* InfiniteAreaLight.cs:21-54 */
    W = map->Width; H = map->Height;
    std::vector<float> lum((size_t)W * H);
    for (int y = 0; y < H; y++) {
        float sinTheta = Sin(((float)y + 0.5f) / (float)H * kPI);
        float v = (float)y / (float)H;
        for (int x = 0; x < W; x++) {
            float u = (float)x / (float)W;
            C3 color = Map->Sample(v2(u, v));
            lum[(size_t)y * W + x] = Luminance(color) * sinTheta;
        }
    }
    Dist = Distribution2D(lum.data(), W, H);
}
void InfiniteAreaLight::Preprocess(const Scene& s) { /* Light.cs:181-187 */
    BBox b = s.Aggregate->WorldBound();
    WorldCenter = b.Center();
    float length = Length(b.Diagonal());
    WorldRadius = length / 2.0f;
}
C3 InfiniteAreaLight::Le(const Ray& ray) const { /* InfiniteAreaLight.cs:56-69 */
    V3 dir = Normalize(TransformNormal(ray.D, WorldToModel));
    float phi = Atan2(dir.x, -dir.z);
    phi = (phi < 0) ? (phi + 2 * kPI) : phi;
    float theta = Acos(netClamp(dir.y, -1, 1));
    float u = phi / (2 * kPI), v = theta / kPI;
    return Map->Sample(v2(u, v));
}
float InfiniteAreaLight::PdfDir(V3 wi) const { /* InfiniteAreaLight.cs:71-85 */
    V3 dir = Normalize(TransformNormal(wi, WorldToModel));
    float phi = Atan2(dir.x, -dir.z);
    phi = (phi < 0) ? (phi + 2 * kPI) : phi;
    float theta = Acos(netClamp(dir.y, -1, 1));
    float sinTheta = Sin(theta);
    if (sinTheta == 0.0f) return 0.0f;
    float u = phi / (2 * kPI), v = theta / kPI;
    return Dist.ContinuousPdf(u, v) / (2 * kPI * kPI * sinTheta);
}
bool InfiniteAreaLight::SampleLightDir(Rng& rand, V2* uv, V3* dirOut, float* pdfOut) const { /* :92-109 */
    float pdf; int ov, ou;
    Dist.SampleContinuous(rand.NextVec2(), &pdf, &ov, &ou);
    if (pdf <= 0) { *uv = v2(0, 0); *dirOut = v3s(0); *pdfOut = 0; return false; }
    float y = (float)ov / (float)H;
    float x = (float)ou / (float)W;
    *uv = v2(x, y);
    float theta = y * kPI;
    float phi = x * 2 * kPI;
    float sinTheta = Sin(theta);
    if (sinTheta == 0) { *dirOut = v3s(0); *pdfOut = 0; return false; }
    pdf /= (2 * kPI * kPI * sinTheta);
    V3 sph = SphericalCoordinates(theta, phi);
    V3 dir = v3(sph.y, sph.z, -sph.x);
    *dirOut = Normalize(TransformNormal(dir, ModelToWorld));
    *pdfOut = pdf;
    return true;
}
SampleLightResult InfiniteAreaLight::SampleLi(LightEvalParam inct, Rng& rand) const { /* :111-119 */
    SampleLightResult r;
    V2 uv; V3 worldDir; float pdfDir;
    SampleLightDir(rand, &uv, &worldDir, &pdfDir);
    if (pdfDir <= 0) return r;
    C3 radiance = Map->Sample(uv);
    V3 pos = worldDir * WorldRadius * 20 + WorldCenter;
    V3 wi = Normalize(pos - inct.P);
    r.P = pos; r.Li = radiance; r.Wi = wi; r.Pdf = pdfDir;
    return r;
}

/* DiffuseAreaLight.SampleEmit (DiffuseAreaLight.cs:70-77) */
LightEmitResult AreaLight::SampleEmit(Rng& rand) const {
    float pdfPos;
    ShapeSurfacePoint samplePoint = S->Sample(rand, &pdfPos);
    V3 localW = Normalize(SquareToCosineHemisphere(rand.NextVec2()));
    float pdfDir = SquareToCosineHemispherePdf(localW);
    V3 w = samplePoint.Shading.ToWorld(localW);
    LightEmitResult r;
    r.Pos = samplePoint.P; r.Dir = Normalize(w); r.Normal = samplePoint.Shading.Z; r.UV = samplePoint.UV;
    r.Radiance = LightEmit; r.PdfPos = pdfPos; r.PdfDir = pdfDir;
    return r;
}
/* InfiniteAreaLight.SampleEmit (InfiniteAreaLight.cs:122-133): a direction from the
 * map's distribution, a position on the disk of the world bounding sphere facing it */
LightEmitResult InfiniteAreaLight::SampleEmit(Rng& rand) const {
    V2 uv; V3 worldDir; float pdfDir;
    SampleLightDir(rand, &uv, &worldDir, &pdfDir);
    C3 radiance = Map->Sample(uv);
    V3 normal = -worldDir;
    Coordinate coord(normal);
    V2 cd = SquareToConcentricDisk(rand.NextVec2());
    V3 disk = WorldCenter + WorldRadius * (cd.x * coord.X + cd.y * coord.Y);
    V3 pos = disk + worldDir * WorldRadius;
    float pdfPos = 1 / (kPI * Sqr(WorldRadius));
    LightEmitResult r;
    r.Pos = pos; r.Dir = -worldDir; r.Normal = -worldDir; r.UV = uv; r.Radiance = radiance;
    r.PdfPos = pdfPos; r.PdfDir = pdfDir;
    return r;
}

/* ---- camera (Camera.cs:182-191) --------------------------------------------------------------- */
Ray PerspectiveCamera::SampleRay(V2 sp) const {
    V3 ndc = v3(sp.x * InvResolve.x, sp.y * InvResolve.y, 0.0f);
    V3 near_ = Transform(ndc, ClipToCamera);
    V3 dir = Normalize(near_);
    float invZ = 1.0f / dir.z;
    V3 o = Transform(v3(0, 0, 0), CameraToWorld);
    V3 d = Normalize(TransformNormal(dir, CameraToWorld));
    return Ray(o, d, Near * invZ, Far * invZ);
}
void PerspectiveCamera::Update() { /* Camera.cs:172-179 */
    V3 pMin = Transform(v3(0, 0, 0), ClipToCamera);
    V3 pMax = Transform(v3(1, 1, 0), ClipToCamera);
    pMin = pMin / pMin.z;
    pMax = pMax / pMax.z;
    Min = v2(pMax.x, pMax.y);
    Max = v2(pMin.x, pMin.y);
    float area = Abs((Max.x - Min.x) * (Max.y - Min.y));
    Normalization = 1 / area;
}
float PerspectiveCamera::Importance(V3 d) const { /* Camera.cs:193-204 */
    float cosTheta = CosTheta(d);
    if (cosTheta <= 0) return 0;
    float focus = 1 / cosTheta;
    V2 p = v2(d.x * focus, d.y * focus);
    if (p.x < Min.x || p.x > Max.x || p.y < Min.y || p.y > Max.y) return 0.0f;
    return Normalization * focus * focus * focus;
}
/* Camera.cs:221-241.  The clip-space point comes from Vector3.Transform (no w
 * divide) and is divided by its own z, the reference's projection as written. */
SampleCameraWiResult PerspectiveCamera::SampleWi(V3 pos) const {
    SampleCameraWiResult r;
    V3 localTarget = Transform(pos, WorldToCamera);
    if (localTarget.z < Near || localTarget.z > Far) return r;
    V3 screen = Transform(localTarget, CameraToClip);
    screen.x = screen.x / screen.z;
    screen.y = screen.y / screen.z;
    screen.z = 1;
    if (screen.x < 0 || screen.x > 1 || screen.y < 0 || screen.y > 1) return r;
    V2 ssPos = v2(screen.x * (float)(ScreenX - 1), screen.y * (float)(ScreenY - 1));
    float dist = Length(localTarget);
    float inv = 1 / dist;
    V3 localDir = localTarget * inv;
    V3 samplePos = Transform(v3(0, 0, 0), CameraToWorld);
    V3 dir = (samplePos - pos) / dist;
    V3 normal = TransformNormal(v3(0, 0, 1), CameraToWorld);
    float importance = Importance(localDir) * inv * inv;
    r.Pos = samplePos; r.Dir = dir; r.Dist = dist; r.Normal = normal; r.Pdf = 1;
    r.We = c3s(importance); r.ScreenPos = ssPos;
    return r;
}

/* ---- scene services (Scene.cs) ------------------------------------------------------------------ */
bool Scene::Intersect(const Ray& ray, Intersection* inct) const {
    if (tl_counters) tl_counters->rays_closest++;
    return Aggregate->Intersect(ray, inct);
}
bool Scene::IntersectP(const Ray& ray) const {
    if (tl_counters) tl_counters->rays_shadow++;
    return Aggregate->IntersectP(ray);
}
C3 Scene::EvalAllInfiniteLights(const Ray& ray) const {
    C3 l = c3s(0.0f);
    for (const InfiniteAreaLight* li : InfiniteLights) l = l + li->Le(ray);
    return l;
}
float Scene::SampleLight(Rng& rand, const Light** light) const {
    if (Lights.empty()) { *light = nullptr; return 0.0f; }
    *light = Lights[rand.Next((int)Lights.size())];
    return 1.0f / (float)Lights.size();
}
bool Scene::IsOccluded(V3 from, V3 to) const {
    V3 vec = to - from;
    float dis = Length(vec);
    if (dis < 0.001f) return true;
    V3 dir = Normalize(vec);
    Ray shadowRay(from, dir, 0.0001f, dis - 0.0001f);
    return IntersectP(shadowRay);
}
/* Both walks below have no bound in the reference; the oracle and the kernels
 * stop after 4096 boundary crossings (never reached by a closed scene). */
static const int kWalkCap = 4096;
C3 Scene::Transmittance(V3 from, V3 to, const Medium* rayEnv, Rng& /*rand*/) const {
    C3 tr = c3s(1.0f);
    V3 start = from;
    V3 dir = Normalize(to - start);
    for (int it = 0; it < kWalkCap; it++) {
        V3 vec = to - start;
        float dis = Length(vec);
        if (dis < 0.0001f) break;
        Ray ray(start, dir, 0.0001f, dis - 0.0001f);
        Intersection inct;
        bool anyHit = Intersect(ray, &inct);
        if (anyHit && inct.HasSurface()) return c3s(0.0f);
        if (rayEnv != nullptr) tr = tr * rayEnv->Tr(ray);
        if (!anyHit) break;
        start = inct.P;
        rayEnv = inct.GetMedium(dir);
    }
    return tr;
}
bool Scene::IntersectTr(Ray ray, const Medium* rayEnv, Rng& /*rand*/, Intersection* inct, C3* tr) const {
    *tr = c3s(1.0f);
    for (int it = 0; it < kWalkCap; it++) {
        bool anyHit = Intersect(ray, inct);
        if (!anyHit) {
            if (rayEnv != nullptr) *tr = *tr * rayEnv->Tr(ray);
            return false;
        }
        if (rayEnv != nullptr) {
            Ray realPath(ray.O, ray.D, ray.MinT, Length(ray.At(inct->T)));
            *tr = *tr * rayEnv->Tr(realPath);
        }
        if (inct->HasSurface()) return true;
        ray = Ray(inct->P, ray.D, 0.001f);
        rayEnv = inct->GetMedium(ray.D);
    }
    return false;
}

/* ---- scene builder (RendererBuilder.Build, RendererBuilder.cs:870-1010) ---------------------------- */
static M44 ToM44(const float* m) { M44 r; memcpy(r.m, m, sizeof(r.m)); return r; }
static std::unique_ptr<TriangleMesh> MakeMesh(const rt_mesh_desc& d) {
    std::unique_ptr<TriangleMesh> m(new TriangleMesh());
    m->Position.resize(d.vertex_count);
    for (int i = 0; i < d.vertex_count; i++) m->Position[i] = v3(d.positions[3 * i], d.positions[3 * i + 1], d.positions[3 * i + 2]);
    if (d.normals) {
        m->Normal.resize(d.vertex_count);
        for (int i = 0; i < d.vertex_count; i++) m->Normal[i] = v3(d.normals[3 * i], d.normals[3 * i + 1], d.normals[3 * i + 2]);
    }
    if (d.uvs) {
        m->UV.resize(d.vertex_count);
        for (int i = 0; i < d.vertex_count; i++) m->UV[i] = v2(d.uvs[2 * i], d.uvs[2 * i + 1]);
    }
    m->Indices.assign(d.indices, d.indices + (size_t)d.triangle_count * 3);
    m->TriangleCount = d.triangle_count;
    return m;
}
std::unique_ptr<Scene> BuildScene(const rt_scene_desc* d, std::string* err) {
    if (!d || d->abi_version != RT_ABI_VERSION) { *err = "bad scene descriptor / ABI version"; return nullptr; }
    std::unique_ptr<Scene> s(new Scene());
    for (int i = 0; i < d->texture_count; i++) {
        const rt_texture_desc& t = d->textures[i];
        if (t.width <= 0 || t.height <= 0 || !t.data) { *err = "bad texture"; return nullptr; }
        std::unique_ptr<Texture2D> tx(new Texture2D());
        tx->Width = t.width; tx->Height = t.height; tx->Wrap = t.wrap; tx->Filter = t.filter;
        tx->data.assign(t.data, t.data + (size_t)t.width * t.height * 3);
        s->textures.push_back(std::move(tx));
    }
    auto tex = [&](int i) -> const Texture2D* { return (i >= 0 && i < (int)s->textures.size()) ? s->textures[i].get() : nullptr; };
    for (int i = 0; i < d->material_count; i++) {
        const rt_material_desc& md = d->materials[i];
        Material m;
        m.type = md.type; m.dist = md.dist; m.twoSided = md.two_sided != 0;
        m.R = tex(md.tex_r); m.T = tex(md.tex_t); m.Rough = tex(md.tex_roughness); m.Anis = tex(md.tex_anisotropic);
        m.etaA = md.eta_a; m.etaB = md.eta_b; m.kd = md.kd; m.ks = md.ks;
        m.Eta = c3(md.eta[0], md.eta[1], md.eta[2]); m.K = c3(md.k[0], md.k[1], md.k[2]);
        bool needR = m.type != RT_MAT_ROUGH_METAL, needT = m.type == RT_MAT_ROUGH_GLASS || m.type == RT_MAT_PERFECT_GLASS;
        bool needRough = m.type == RT_MAT_ROUGH_METAL || m.type == RT_MAT_ROUGH_GLASS || m.type == RT_MAT_ROUGH_PLASTIC;
        if ((needR && !m.R) || (needT && !m.T) || (needRough && (!m.Rough || !m.Anis)) || m.type < 0 || m.type > 5) {
            *err = "material " + std::to_string(i) + " is missing a texture or has an unknown type"; return nullptr;
        }
        s->materials.push_back(m);
    }
    for (int i = 0; i < d->medium_count; i++) {
        const rt_medium_desc& md = d->media[i];
        Medium m;
        m.SigmaA = c3(md.sigma_a[0], md.sigma_a[1], md.sigma_a[2]) * md.scale;
        m.SigmaS = c3(md.sigma_s[0], md.sigma_s[1], md.sigma_s[2]) * md.scale;
        m.SigmaT = m.SigmaA + m.SigmaS;
        m.G = md.g;
        s->media.push_back(m);
    }
    auto med = [&](int i) -> const Medium* { return (i >= 0 && i < (int)s->media.size()) ? &s->media[i] : nullptr; };
    auto mat = [&](int i) -> const Material* { return (i >= 0 && i < (int)s->materials.size()) ? &s->materials[i] : nullptr; };
    for (int i = 0; i < d->mesh_count; i++) s->meshes.push_back(MakeMesh(d->meshes[i]));
    auto sphere = [&](int i) -> const Shape* {
        const rt_sphere_desc& sd = d->spheres[i];
        s->shapes.emplace_back(new Sphere(sd.radius, v3(sd.center[0], sd.center[1], sd.center[2]), ToM44(sd.model_to_world), ToM44(sd.world_to_model)));
        return s->shapes.back().get();
    };
    /* instanced prototypes: ShapeWrapperPrimitive per shape, own Bvh */
    for (int b = 0; b < d->blas_count; b++) {
        int first = d->blas_ranges[2 * b], count = d->blas_ranges[2 * b + 1];
        std::vector<const Primitive*> prims;
        for (int g = first; g < first + count; g++) {
            const rt_group_desc& gd = d->blas_groups[g];
            if (gd.kind == RT_GROUP_SPHERE) {
                const Shape* sh = sphere(gd.ref);
                s->primStore.emplace_back(new ShapeWrapperPrimitive(sh));
                s->primStore.back()->id = (int)prims.size();
                prims.push_back(s->primStore.back().get());
            } else if (gd.kind == RT_GROUP_MESH) {
                const TriangleMesh* m = s->meshes[gd.ref].get();
                for (int t = 0; t < m->TriangleCount; t++) {
                    s->shapes.emplace_back(new Triangle(m, t));
                    s->primStore.emplace_back(new ShapeWrapperPrimitive(s->shapes.back().get()));
                    s->primStore.back()->id = (int)prims.size();
                    prims.push_back(s->primStore.back().get());
                }
            } else { *err = "instanced prototype group must be a mesh or a sphere"; return nullptr; }
        }
        s->blas.emplace_back(new Bvh(prims, d->bvh_max_prims));
    }
    std::vector<const Primitive*> prims;
    for (int g = 0; g < d->group_count; g++) {
        const rt_group_desc& gd = d->groups[g];
        MediumAdapter ma; ma.Inside = med(gd.medium_inside); ma.Outside = med(gd.medium_outside);
        C3 le = c3(gd.le[0], gd.le[1], gd.le[2]);
        auto addGeom = [&](const Shape* sh) {
            GeometricPrimitive* gp = new GeometricPrimitive(sh, mat(gd.material), ma);
            s->primStore.emplace_back(gp);
            gp->id = (int)prims.size();
            if (gd.emissive) {
                AreaLight* al = new AreaLight(sh, le);
                al->index = (int)s->Lights.size();
                s->lightStore.emplace_back(al);
                s->Lights.push_back(al);
                gp->Lt = al;
            }
            prims.push_back(gp);
        };
        switch (gd.kind) {
        case RT_GROUP_INFINITE_LIGHT: {
            InfiniteAreaLight* il = new InfiniteAreaLight(ToM44(gd.model_to_world), ToM44(gd.world_to_model), tex(gd.ref));
            il->index = (int)s->Lights.size();
            s->lightStore.emplace_back(il);
            s->Lights.push_back(il);
            s->InfiniteLights.push_back(il);
            break;
        }
        case RT_GROUP_SPHERE: addGeom(sphere(gd.ref)); break;
        case RT_GROUP_MESH: {
            const TriangleMesh* m = s->meshes[gd.ref].get();
            for (int t = 0; t < m->TriangleCount; t++) {
                s->shapes.emplace_back(new Triangle(m, t));
                addGeom(s->shapes.back().get());
            }
            break;
        }
        case RT_GROUP_INSTANCE: {
            InstancedPrimitive* ip = new InstancedPrimitive(s->blas[gd.ref].get(), ToM44(gd.model_to_world), ToM44(gd.world_to_model), mat(gd.material), ma);
            s->primStore.emplace_back(ip);
            ip->id = (int)prims.size();
            prims.push_back(ip);
            break;
        }
        default: *err = "unknown group kind"; return nullptr;
        }
    }
    if (prims.empty()) { *err = "scene has no primitives"; return nullptr; }
    s->Aggregate.reset(new Bvh(prims, d->bvh_max_prims));
    s->GlobalMedium = med(d->global_medium);
    const rt_camera_desc& c = d->camera;
    s->Camera.ScreenX = c.width; s->Camera.ScreenY = c.height; s->Camera.Near = c.near_z; s->Camera.Far = c.far_z;
    s->Camera.ClipToCamera = ToM44(c.clip_to_camera); s->Camera.CameraToWorld = ToM44(c.camera_to_world);
    s->Camera.InvResolve = v2(1.0f / (float)c.width, 1.0f / (float)c.height);
    s->Camera.CameraToClip = ToM44(c.camera_to_clip); s->Camera.WorldToCamera = ToM44(c.world_to_camera);
    s->Camera.Update();
    for (InfiniteAreaLight* il : s->InfiniteLights) il->Preprocess(*s);
    return s;
}

} /* namespace orc */
