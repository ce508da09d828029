/*
 * or_scene.h - CPU oracle, part 2: the reference's plugin types.
 *
 * TEST INFRASTRUCTURE ONLY (see or_core.h).  Class-for-class restatement of
 * Radiantium.Offline: Shape/Primitive/Bvh, Material + BxDFs, Light, Medium,
 * Texture2D, Camera and Scene.  File:line citations name the C# source each
 * piece follows.
 */
#ifndef OR_SCENE_H
#define OR_SCENE_H

#include <vector>
#include <memory>
#include "or_core.h"
#include "../include/radiantium.h"

namespace orc {

struct Primitive;
struct Material;
struct AreaLight;
struct Medium;

/* per-thread traversal counters (algorithmic bytes of the roofline) */
struct Counters {
    uint64_t node_visits = 0, prim_tests = 0, instance_visits = 0;
    uint64_t rays_closest = 0, rays_shadow = 0;
};
extern thread_local Counters* tl_counters;

/* Intersection.cs:5-16 */
struct SurfacePoint { float U, V, T; };

/* Shape.cs:5-40 */
struct ShapeIntersection { V3 P; V2 UV; float T; Coordinate Shading; V3 Wr; };
struct ShapeSurfacePoint { V3 P; V2 UV; Coordinate Shading; };

/* Intersection.cs:18-72 */
struct Intersection {
    V3 P; V2 UV; float T = 0; const Primitive* Shape = nullptr; Coordinate Shading; V3 Wr;
    int prim_id = -1, sub_id = -1; /* parity bookkeeping, not in the reference */
    float bu = 0, bv = 0;          /* SurfacePoint U, V of the hit triangle */
    uint32_t flags = 0;
    V3 N() const { return Shading.Z; }
    bool IsLight() const;
    const AreaLight* Light() const;
    bool HasSurface() const;
    const Material* Surface() const;
    Ray SpawnRay(V3 d) const { return Ray(P, d, 0.0001f); }
    C3 Le(V3 w) const;
    V3 ToLocal(V3 v) const { return Shading.ToLocal(v); }
    V3 ToWorld(V3 v) const { return Shading.ToWorld(v); }
    const Medium* GetMedium(V3 w) const;
};

/* ---- textures: Texture2D.cs, TextureSampler.cs, Textures/ --------------- */
struct Texture2D {
    int Width = 1, Height = 1, Wrap = RT_WRAP_CLAMP, Filter = RT_FILTER_NEAREST;
    std::vector<float> data; /* ColorBuffer layout */
    C3 Read(int x, int y) const {
        /* ColorBuffer.GetIndex throws on out-of-range indices; the only way to
         * get there is a NaN uv, which the oracle clamps instead. */
        x = netClampI(x, 0, Width - 1); y = netClampI(y, 0, Height - 1);
        const float* p = &data[((size_t)x * Height + y) * 3];
        return c3(p[0], p[1], p[2]);
    }
    C3 Sample(V2 uv) const { return Sample(uv.x, uv.y); }
    C3 Sample(float x, float y) const;
};

/* ---- shapes ----------------------------------------------------------------- */
struct Shape {
    BBox WorldBound;
    virtual ~Shape() {}
    virtual float SurfaceArea() const = 0;
    virtual bool IntersectP(const Ray& ray) const = 0;
    virtual bool Intersect(const Ray& ray, SurfacePoint* sp) const = 0;
    virtual ShapeIntersection GetIntersection(const Ray& ray, SurfacePoint sp) const = 0;
    virtual ShapeSurfacePoint Sample(Rng& rand, float* pdf) const = 0;
    virtual float Pdf(const ShapeSurfacePoint&) const = 0;
};

/* Shapes/Triangle.cs:6-62 */
struct TriangleMesh {
    std::vector<V3> Position, Normal;
    std::vector<V2> UV;
    std::vector<int> Indices;
    int TriangleCount = 0;
    bool HasNormal() const { return !Normal.empty(); }
    bool HasUV() const { return !UV.empty(); }
};

/* Shapes/Triangle.cs:65-213 */
struct Triangle : Shape {
    const TriangleMesh* Mesh; int Index; float Area;
    Triangle(const TriangleMesh* m, int i);
    const V3& Pa() const { return Mesh->Position[Mesh->Indices[Index * 3 + 0]]; }
    const V3& Pb() const { return Mesh->Position[Mesh->Indices[Index * 3 + 1]]; }
    const V3& Pc() const { return Mesh->Position[Mesh->Indices[Index * 3 + 2]]; }
    float SurfaceArea() const override { return Area; }
    bool IntersectP(const Ray& ray) const override;
    bool Intersect(const Ray& ray, SurfacePoint* sp) const override;
    ShapeIntersection GetIntersection(const Ray& ray, SurfacePoint sp) const override;
    ShapeSurfacePoint Sample(Rng& rand, float* pdf) const override;
    float Pdf(const ShapeSurfacePoint&) const override { return 1.0f / Area; }
};

/* Shapes/Sphere.cs */
struct Sphere : Shape {
    float Radius; V3 Center; M44 ModelToWorld, WorldToModel;
    Sphere(float r, V3 c, const M44& m2w, const M44& w2m);
    float SurfaceArea() const override { return 4 * Radius * Radius * kPI; }
    bool IntersectP(const Ray& ray) const override;
    bool Intersect(const Ray& ray, SurfacePoint* sp) const override;
    ShapeIntersection GetIntersection(const Ray& ray, SurfacePoint sp) const override;
    ShapeSurfacePoint Sample(Rng& rand, float* pdf) const override;
    float Pdf(const ShapeSurfacePoint&) const override { return 1 / SurfaceArea(); }
};

/* ---- media: Medium.cs, Mediums/Homogeneous.cs, IPhaseFunction.cs ---------------- */
struct MediumAdapter { const Medium* Inside = nullptr; const Medium* Outside = nullptr; };
struct SampleMediumResult {
    const Medium* M = nullptr; V3 P; V3 Wo; C3 Tr; float T = 0; bool IsSampleMedium = false;
};
struct SamplePhaseFunctionResult { float P; V3 Wi; };
struct Medium {
    C3 SigmaA, SigmaS, SigmaT; float G; /* HG g as given (clamped by HenyeyGreenstein) */
    C3 Tr(const Ray& ray) const;
    SampleMediumResult Sample(const Ray& ray, Rng& rand) const;
    float P(V3 wo, V3 wi) const;
    SamplePhaseFunctionResult SampleWi(V3 wo, Rng& rand) const;
};

/* ---- primitives: Primitive.cs ------------------------------------------------ */
struct Primitive {
    int id = -1; /* index in the owner's primitive list */
    virtual ~Primitive() {}
    virtual const Material* GetMaterial() const { return nullptr; }
    virtual const AreaLight* GetLight() const { return nullptr; }
    virtual BBox WorldBound() const = 0;
    virtual const MediumAdapter* GetMedium() const { return nullptr; }
    virtual bool IntersectP(const Ray& ray) const = 0;
    virtual bool Intersect(const Ray& ray, Intersection* inct) const = 0;
};

struct GeometricPrimitive : Primitive {
    const Shape* S; const Material* Mat; const AreaLight* Lt = nullptr; MediumAdapter Med;
    GeometricPrimitive(const Shape* s, const Material* m, MediumAdapter med) : S(s), Mat(m), Med(med) {}
    const Material* GetMaterial() const override { return Mat; }
    const AreaLight* GetLight() const override { return Lt; }
    BBox WorldBound() const override { return S->WorldBound; }
    const MediumAdapter* GetMedium() const override { return &Med; }
    bool IntersectP(const Ray& ray) const override;
    bool Intersect(const Ray& ray, Intersection* inct) const override;
};

struct ShapeWrapperPrimitive : Primitive {
    const Shape* S;
    explicit ShapeWrapperPrimitive(const Shape* s) : S(s) {}
    BBox WorldBound() const override { return S->WorldBound; }
    bool IntersectP(const Ray& ray) const override;
    bool Intersect(const Ray& ray, Intersection* inct) const override;
};

/* Accelerators/Bvh.cs */
struct LinearBVHNode { BBox Bounds; int PrimitivesIndex; /* or SecondChildIndex */ uint16_t PrimitiveCount; uint8_t Axis; };
struct Bvh : Primitive {
    std::vector<const Primitive*> prims;  /* ordered primitives */
    std::vector<LinearBVHNode> nodes;
    int maxPrims;
    int leafCount = 0;
    Bvh(const std::vector<const Primitive*>& p, int maxPrimsInNode);
    BBox WorldBound() const override { return nodes.empty() ? BBox() : nodes[0].Bounds; }
    bool IntersectP(const Ray& ray) const override;
    bool Intersect(const Ray& ray, Intersection* inct) const override;
};

struct InstancedPrimitive : Primitive {
    const Primitive* Instanced; M44 ModelToWorld, WorldToModel; const Material* Mat; MediumAdapter Med; BBox Bound;
    InstancedPrimitive(const Primitive* inst, const M44& m2w, const M44& w2m, const Material* m, MediumAdapter med);
    const Material* GetMaterial() const override { return Mat; }
    BBox WorldBound() const override { return Bound; }
    const MediumAdapter* GetMedium() const override { return &Med; }
    bool IntersectP(const Ray& ray) const override;
    bool Intersect(const Ray& ray, Intersection* inct) const override;
};

/* ---- materials: Material.cs, IBxdf.cs, Materials/, Bxdf/ ---------------------- */
enum BxdfType { Reflection = 1, Transmission = 2, Diffuse_ = 4, Glossy = 8, Specular = 16 };
struct SampleBxdfResult { V3 Wi = v3s(0); C3 Fr = c3s(0); float Pdf = 0; int Type = 0; };

struct Material {
    int type; int dist; bool twoSided;
    const Texture2D *R = nullptr, *T = nullptr, *Rough = nullptr, *Anis = nullptr;
    float etaA = 1, etaB = 1, kd = 0.5f, ks = 0.5f;
    C3 Eta, K;
    /* importance: TransportMode.Importance instead of Radiance */
    C3 Fr(V3 wo, V3 wi, const Intersection& inct, bool importance = false) const;
    float Pdf(V3 wo, V3 wi, const Intersection& inct) const;
    SampleBxdfResult Sample(V3 wo, const Intersection& inct, Rng& rand, bool importance = false) const;
};

/* ---- lights: Light.cs, Lights/ -------------------------------------------- */
struct SampleLightResult { V3 P = v3s(0); C3 Li = c3s(0); V3 Wi = v3s(0); float Pdf = 0; };
struct LightEvalParam { V3 P; float T; };
/* Light.cs:61-107 LightEmitResult + LightEmitPdf */
struct LightEmitResult {
    V3 Pos = v3s(0), Dir = v3s(0), Normal = v3s(0); V2 UV = v2(0, 0); C3 Radiance = c3s(0);
    float PdfPos = 0, PdfDir = 0;
};
struct Scene;
struct Light {
    int index = -1;
    virtual ~Light() {}
    bool IsDelta() const { return false; } /* Area and Infinite lights are never delta */
    virtual SampleLightResult SampleLi(LightEvalParam inct, Rng& rand) const = 0;
    virtual float PdfLi(LightEvalParam inct, V3 wi) const = 0;
    virtual LightEmitResult SampleEmit(Rng& rand) const = 0;
    virtual C3 Le(const Ray&) const { return c3s(0); }
};
struct AreaLight : Light {
    C3 LightEmit; const Shape* S; float Area;
    AreaLight(const Shape* s, C3 le) : LightEmit(le), S(s), Area(s->SurfaceArea()) {}
    C3 L(const Intersection& inct, V3 w) const { return (Dot(inct.N(), w) > 0) ? LightEmit : c3s(0); }
    SampleLightResult SampleLi(LightEvalParam inct, Rng& rand) const override;
    float PdfLi(LightEvalParam inct, V3 wi) const override;
    LightEmitResult SampleEmit(Rng& rand) const override;
};
/* Distribution1D.cs / Distribution2D.cs */
struct Distribution1D {
    std::vector<float> pdf, cdf; float integration = 0;
    Distribution1D() {}
    explicit Distribution1D(const float* p, int n);
    int Count() const { return (int)pdf.size(); }
    int FindInterval(float u) const;
    float SampleContinuous(float u, float* pdfOut, int* offset) const;
    float ContinuousPdf(int offset) const { return integration > 0 ? pdf[offset] / integration : 0; }
};
struct Distribution2D {
    std::vector<Distribution1D> conditional; Distribution1D marginal;
    Distribution2D() {}
    Distribution2D(const float* data, int nu, int nv);
    V2 SampleContinuous(V2 u, float* pdf, int* offV, int* offU) const;
    float ContinuousPdf(float u, float v) const;
};
struct InfiniteAreaLight : Light {
    M44 ModelToWorld, WorldToModel; const Texture2D* Map; Distribution2D Dist; int W, H;
    float WorldRadius = 0; V3 WorldCenter = v3s(0);
    InfiniteAreaLight(const M44& m2w, const M44& w2m, const Texture2D* map);
    void Preprocess(const Scene& s);
    C3 Le(const Ray& ray) const override;
    float PdfDir(V3 wi) const;
    float PdfLi(LightEvalParam, V3 wi) const override { return PdfDir(wi); }
    bool SampleLightDir(Rng& rand, V2* uv, V3* dir, float* pdf) const;
    SampleLightResult SampleLi(LightEvalParam inct, Rng& rand) const override;
    LightEmitResult SampleEmit(Rng& rand) const override;
};

/* ---- camera: Camera.cs PerspectiveCamera ---------------------------------------- */
/* Camera.cs:21-48 SampleCameraWiResult */
struct SampleCameraWiResult {
    V3 Pos = v3s(0), Dir = v3s(0); float Dist = 0; V3 Normal = v3s(0); float Pdf = 0; C3 We = c3s(0);
    V2 ScreenPos = v2(0, 0);
};
struct PerspectiveCamera {
    int ScreenX, ScreenY; float Near, Far; M44 ClipToCamera, CameraToWorld; V2 InvResolve;
    M44 CameraToClip, WorldToCamera; V2 Min, Max; float Normalization;
    void Update(); /* the _min/_max/_normalization part of Update (Camera.cs:172-179) */
    Ray SampleRay(V2 samplePosition) const;
    float Importance(V3 d) const;
    SampleCameraWiResult SampleWi(V3 pos) const;
};

/* ---- scene: Scene.cs ------------------------------------------------------------ */
struct Scene {
    /* storage */
    std::vector<std::unique_ptr<TriangleMesh>> meshes, blasMeshes;
    std::vector<std::unique_ptr<Shape>> shapes;
    std::vector<std::unique_ptr<Primitive>> primStore;
    std::vector<std::unique_ptr<Texture2D>> textures;
    std::vector<Material> materials;
    std::vector<Medium> media;
    std::vector<std::unique_ptr<Bvh>> blas;
    std::vector<std::unique_ptr<Light>> lightStore;
    /* Scene.cs:8-12 */
    std::unique_ptr<Bvh> Aggregate;
    std::vector<const Light*> Lights;
    std::vector<InfiniteAreaLight*> InfiniteLights;
    const Medium* GlobalMedium = nullptr;
    PerspectiveCamera Camera;

    bool Intersect(const Ray& ray, Intersection* inct) const;
    bool IntersectP(const Ray& ray) const;
    C3 EvalAllInfiniteLights(const Ray& ray) const;
    float SampleLight(Rng& rand, const Light** light) const;
    bool IsOccluded(V3 from, V3 to) const;
    C3 Transmittance(V3 from, V3 to, const Medium* rayEnv, Rng& rand) const;
    bool IntersectTr(Ray ray, const Medium* rayEnv, Rng& rand, Intersection* inct, C3* tr) const;
};

/* builds the oracle scene from the flattened description; returns an error message or "" */
std::unique_ptr<Scene> BuildScene(const rt_scene_desc* d, std::string* err);

/* integrators */
C3 PathLi(const Scene& s, const rt_render_params& p, Ray ray, Rng& rand);
C3 VolPathLi(const Scene& s, const rt_render_params& p, Ray ray, Rng& rand);
/* AdjointParticleIntegrator.EmitParticle: calls splat(x, y, color) per camera connection */
struct Splat { int x, y; C3 color; };
void EmitParticle(const Scene& s, const rt_render_params& p, Rng& rand, std::vector<Splat>* splats);
C3 CameraTraceLight(const Scene& s, const Ray& ray);

} /* namespace orc */

#endif
