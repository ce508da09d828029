"""Flattened scene description (the host-side counterpart of rt_scene_desc).

A :class:`SceneDesc` is what the reference's ``RendererBuilder.Build`` produces
once its Scene is walked: world-space triangle meshes, spheres, instanced
prototypes, textures, material/medium tables, entity groups in build order and
the perspective camera.  ``to_c`` packs it into the C structures of
include/radiantium.h.

Matrix arithmetic follows System.Numerics.Matrix4x4 (row vectors, float32 and
the operation order of the reference's call sites); every intermediate value
is rounded to float32 as the .NET JIT does.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import native as N

F = np.float32


# ---------------------------------------------------------------- Matrix4x4 ----
class Mat4:
    """A System.Numerics.Matrix4x4 (M11..M44, row vectors) with float32 arithmetic."""

    __slots__ = ("m",)

    def __init__(self, m=None):
        self.m = [F(0)] * 16 if m is None else [F(v) for v in m]

    @staticmethod
    def identity():
        return Mat4([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1])

    @staticmethod
    def translation(p):
        r = Mat4.identity()
        r.m[12], r.m[13], r.m[14] = F(p[0]), F(p[1]), F(p[2])
        return r

    @staticmethod
    def scale(s):
        r = Mat4.identity()
        r.m[0], r.m[5], r.m[10] = F(s[0]), F(s[1]), F(s[2])
        return r

    @staticmethod
    def from_axis_angle(axis, angle_rad):
        """Matrix4x4.CreateFromAxisAngle: Rodrigues' rotation formula for row vectors."""
        x, y, z = (F(a) for a in axis)
        a = F(angle_rad)
        sa, ca = F(math.sin(float(a))), F(math.cos(float(a)))
        xx, yy, zz = x * x, y * y, z * z
        xy, xz, yz = x * y, x * z, y * z
        one = F(1)
        r = Mat4.identity()
        r.m[0] = xx + ca * (one - xx)
        r.m[1] = xy - ca * xy + sa * z
        r.m[2] = xz - ca * xz - sa * y
        r.m[4] = xy - ca * xy - sa * z
        r.m[5] = yy + ca * (one - yy)
        r.m[6] = yz - ca * yz + sa * x
        r.m[8] = xz - ca * xz + sa * y
        r.m[9] = yz - ca * yz - sa * x
        r.m[10] = zz + ca * (one - zz)
        return r

    def __mul__(self, o: "Mat4") -> "Mat4":
        a, b = self.m, o.m
        r = Mat4()
        for i in range(4):
            for j in range(4):
                acc = a[4 * i] * b[j]
                acc = acc + a[4 * i + 1] * b[4 + j]
                acc = acc + a[4 * i + 2] * b[8 + j]
                acc = acc + a[4 * i + 3] * b[12 + j]
                r.m[4 * i + j] = F(acc)
        return r

    def invert(self) -> "Mat4":
        """4x4 inverse by cofactor (Laplace) expansion in float32; raises if singular
        (Matrix4x4.Invert returning false is an ArgumentException in the reference)."""
        a, b, c, d, e, f, g, h, i, j, k, l, mm, n, o, p = self.m
        kp_lo = k * p - l * o
        jp_ln = j * p - l * n
        jo_kn = j * o - k * n
        ip_lm = i * p - l * mm
        io_km = i * o - k * mm
        in_jm = i * n - j * mm
        a11 = f * kp_lo - g * jp_ln + h * jo_kn
        a12 = -(e * kp_lo - g * ip_lm + h * io_km)
        a13 = e * jp_ln - f * ip_lm + h * in_jm
        a14 = -(e * jo_kn - f * io_km + g * in_jm)
        det = a * a11 + b * a12 + c * a13 + d * a14
        if abs(float(det)) < 1.401298464324817e-45:
            raise ValueError("invalid transform matrix (singular)")
        inv = F(1) / det
        gp_ho = g * p - h * o
        fp_hn = f * p - h * n
        fo_gn = f * o - g * n
        ep_hm = e * p - h * mm
        eo_gm = e * o - g * mm
        en_fm = e * n - f * mm
        gl_hk = g * l - h * k
        fl_hj = f * l - h * j
        fk_gj = f * k - g * j
        el_hi = e * l - h * i
        ek_gi = e * k - g * i
        ej_fi = e * j - f * i
        r = Mat4()
        r.m = [a11 * inv, -(b * kp_lo - c * jp_ln + d * jo_kn) * inv, (b * gp_ho - c * fp_hn + d * fo_gn) * inv,
               -(b * gl_hk - c * fl_hj + d * fk_gj) * inv,
               a12 * inv, (a * kp_lo - c * ip_lm + d * io_km) * inv, -(a * gp_ho - c * ep_hm + d * eo_gm) * inv,
               (a * gl_hk - c * el_hi + d * ek_gi) * inv,
               a13 * inv, -(a * jp_ln - b * ip_lm + d * in_jm) * inv, (a * fp_hn - b * ep_hm + d * en_fm) * inv,
               -(a * fl_hj - b * el_hi + d * ej_fi) * inv,
               a14 * inv, (a * jo_kn - b * io_km + c * in_jm) * inv, -(a * fo_gn - b * eo_gm + c * en_fm) * inv,
               (a * fk_gj - b * ek_gi + c * ej_fi) * inv]
        r.m = [F(v) for v in r.m]
        return r

    def is_identity(self):
        return all(float(self.m[q]) == (1.0 if q % 5 == 0 else 0.0) for q in range(16))

    def array(self):
        return np.array(self.m, dtype=np.float32)


def transform_points(p: np.ndarray, m: Mat4) -> np.ndarray:
    """Vector3.Transform over an (n,3) float32 array: x*M11 + y*M21 + z*M31 + M41, left to right."""
    p = np.asarray(p, dtype=np.float32)
    M = m.m
    out = np.empty_like(p)
    for c in range(3):
        acc = p[:, 0] * M[c]
        acc = acc + p[:, 1] * M[4 + c]
        acc = acc + p[:, 2] * M[8 + c]
        out[:, c] = acc + M[12 + c]
    return out


def transform_normals(v: np.ndarray, m: Mat4) -> np.ndarray:
    """Vector3.TransformNormal over an (n,3) float32 array (no translation, no renormalisation)."""
    v = np.asarray(v, dtype=np.float32)
    M = m.m
    out = np.empty_like(v)
    for c in range(3):
        acc = v[:, 0] * M[c]
        acc = acc + v[:, 1] * M[4 + c]
        out[:, c] = acc + v[:, 2] * M[8 + c]
    return out


def _v3_normalize(v):
    v = [F(a) for a in v]
    ln = F(np.sqrt(F(v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]))
    return [v[0] / ln, v[1] / ln, v[2] / ln]


def _v3_cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


def look_at_left_hand(origin, target, up) -> Mat4:
    """MathExt.LookAtLeftHand (Radiantium.Core/MathExt.cs:148-160): camera->world."""
    o = [F(x) for x in origin]
    t = [F(x) for x in target]
    d = _v3_normalize([t[0] - o[0], t[1] - o[1], t[2] - o[2]])
    left = _v3_normalize(_v3_cross(_v3_normalize(up), d))
    real_up = _v3_normalize(_v3_cross(d, left))
    return Mat4([left[0], left[1], left[2], 0, real_up[0], real_up[1], real_up[2], 0,
                 d[0], d[1], d[2], 0, o[0], o[1], o[2], 1])


@dataclass
class Camera:
    """PerspectiveCamera (Camera.cs:79-162)."""
    width: int
    height: int
    fov: float = 60.0
    near: float = 0.001
    far: float = 1000.0
    camera_to_world: Mat4 = field(default_factory=Mat4.identity)

    @staticmethod
    def look_at(width, height, fov, origin, target, up=(0, 1, 0), near=0.001, far=1000.0):
        return Camera(width, height, fov, near, far, look_at_left_hand(origin, target, up))

    def camera_to_clip(self) -> Mat4:
        """Update(): perspective * translate * scale (Camera.cs:128-159)."""
        near, far = F(self.near), F(self.far)
        aspect = F(self.width) / F(self.height)
        recip = F(1) / (far - near)
        half = F(F(self.fov) / F(2))
        rad = half * (F(3.14159265) / F(180))
        cot = F(1) / F(math.tan(float(rad)))
        persp = Mat4([cot, 0, 0, 0, 0, cot, 0, 0, 0, 0, far * recip, 1, 0, 0, -near * far * recip, 0])
        scale = Mat4([F(-0.5), 0, 0, 0, 0, F(-0.5) * aspect, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1])
        trans = Mat4([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, -1, F(-1) / aspect, 0, 1])
        return (persp * trans) * scale

    def clip_to_camera(self) -> Mat4:
        """Update(): Matrix4x4.Invert of camera->clip (Camera.cs:161-164)."""
        return self.camera_to_clip().invert()

    def world_to_camera(self) -> Mat4:
        """Update(): Matrix4x4.Invert of camera->world (Camera.cs:166-170)."""
        return self.camera_to_world.invert()


# ---------------------------------------------------------------- scene tables ----
@dataclass
class Mesh:
    positions: np.ndarray            # (n,3) float32
    indices: np.ndarray              # (t,3) int32
    normals: np.ndarray | None = None
    uvs: np.ndarray | None = None

    def __post_init__(self):
        self.positions = np.ascontiguousarray(self.positions, dtype=np.float32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(self.indices, dtype=np.int32).reshape(-1, 3)
        if self.normals is not None:
            self.normals = np.ascontiguousarray(self.normals, dtype=np.float32).reshape(-1, 3)
        if self.uvs is not None:
            self.uvs = np.ascontiguousarray(self.uvs, dtype=np.float32).reshape(-1, 2)

    @property
    def triangle_count(self):
        return int(self.indices.shape[0])

    def transformed(self, m: Mat4) -> "Mesh":
        """TriangleMesh(modelToWorld, model) (Shapes/Triangle.cs:15-51)."""
        if m.is_identity():
            return Mesh(self.positions.copy(), self.indices, None if self.normals is None else self.normals.copy(),
                        self.uvs)
        return Mesh(transform_points(self.positions, m), self.indices,
                    None if self.normals is None else transform_normals(self.normals, m), self.uvs)


@dataclass
class Texture:
    """ConstColorTexture2D (1x1) or ImageTexture2D; data in ColorBuffer layout (x*h + y)*3."""
    width: int
    height: int
    data: np.ndarray
    wrap: int = N.WRAP_CLAMP
    filter: int = N.FILTER_NEAREST

    @staticmethod
    def const(rgb):
        c = np.asarray(rgb, dtype=np.float32)
        if c.size == 1:
            c = np.repeat(c, 3)
        return Texture(1, 1, c.reshape(3).copy())

    @staticmethod
    def from_image_hw3(img: np.ndarray, wrap=N.WRAP_CLAMP, filt=N.FILTER_NEAREST):
        """img[y, x, c] -> ColorBuffer layout."""
        img = np.asarray(img, dtype=np.float32)
        h, w, _ = img.shape
        return Texture(w, h, np.ascontiguousarray(img.transpose(1, 0, 2)).reshape(-1), wrap, filt)


@dataclass
class Material:
    type: int
    dist: int = N.DIST_GGX
    two_sided: bool = False
    tex_r: int = -1
    tex_t: int = -1
    tex_roughness: int = -1
    tex_anisotropic: int = -1
    eta_a: float = 1.000277
    eta_b: float = 1.5046
    kd: float = 0.5
    ks: float = 0.5
    eta: tuple = (0.0, 0.0, 0.0)
    k: tuple = (0.0, 0.0, 0.0)


@dataclass
class Medium:
    sigma_a: tuple
    sigma_s: tuple
    g: float = 0.0
    scale: float = 1.0


@dataclass
class Sphere:
    center: tuple
    radius: float
    model_to_world: Mat4 = field(default_factory=Mat4.identity)


@dataclass
class Group:
    kind: int
    ref: int
    material: int = -1
    medium_inside: int = -1
    medium_outside: int = -1
    emissive: bool = False
    le: tuple = (0.0, 0.0, 0.0)
    model_to_world: Mat4 = field(default_factory=Mat4.identity)


@dataclass
class SceneDesc:
    camera: Camera
    meshes: list = field(default_factory=list)
    spheres: list = field(default_factory=list)
    textures: list = field(default_factory=list)
    materials: list = field(default_factory=list)
    media: list = field(default_factory=list)
    blas: list = field(default_factory=list)      # list of lists of Group (MESH / SPHERE)
    groups: list = field(default_factory=list)
    global_medium: int = -1
    bvh_max_prims: int = 1
    name: str = ""

    # -- table helpers ------------------------------------------------------
    def add_texture(self, t: Texture) -> int:
        self.textures.append(t)
        return len(self.textures) - 1

    def add_const(self, rgb) -> int:
        return self.add_texture(Texture.const(rgb))

    def add_material(self, m: Material) -> int:
        self.materials.append(m)
        return len(self.materials) - 1

    def add_mesh(self, m: Mesh) -> int:
        self.meshes.append(m)
        return len(self.meshes) - 1

    def add_medium(self, m: Medium) -> int:
        self.media.append(m)
        return len(self.media) - 1

    @property
    def triangle_count(self) -> int:
        n = 0
        for g in self.groups:
            if g.kind == N.GROUP_MESH:
                n += self.meshes[g.ref].triangle_count
            elif g.kind == N.GROUP_INSTANCE:
                n += sum(self.meshes[b.ref].triangle_count for b in self.blas[g.ref] if b.kind == N.GROUP_MESH)
        return n

    # -- packing --------------------------------------------------------------
    def to_c(self) -> "PackedScene":
        return PackedScene(self)


def _fp(a):
    return a.ctypes.data_as(N.FloatP) if a is not None else N.FloatP()


class PackedScene:
    """Holds the ctypes structures and keeps every numpy buffer alive."""

    def __init__(self, s: SceneDesc):
        keep = []
        meshes = (N.MeshDesc * max(1, len(s.meshes)))()
        for i, m in enumerate(s.meshes):
            keep.append(m)
            meshes[i].vertex_count = m.positions.shape[0]
            meshes[i].triangle_count = m.triangle_count
            meshes[i].positions = _fp(m.positions)
            meshes[i].normals = _fp(m.normals)
            meshes[i].uvs = _fp(m.uvs)
            meshes[i].indices = m.indices.ctypes.data_as(N.IntP)
        spheres = (N.SphereDesc * max(1, len(s.spheres)))()
        for i, sp in enumerate(s.spheres):
            spheres[i].center[:] = [float(F(c)) for c in sp.center]
            spheres[i].radius = float(F(sp.radius))
            spheres[i].model_to_world[:] = [float(v) for v in sp.model_to_world.m]
            spheres[i].world_to_model[:] = [float(v) for v in sp.model_to_world.invert().m]
        textures = (N.TextureDesc * max(1, len(s.textures)))()
        for i, t in enumerate(s.textures):
            d = np.ascontiguousarray(t.data, dtype=np.float32)
            if d.size != t.width * t.height * 3:
                raise ValueError(f"texture {i}: data size {d.size} != {t.width}x{t.height}x3")
            keep.append(d)
            textures[i].width, textures[i].height = t.width, t.height
            textures[i].wrap, textures[i].filter = t.wrap, t.filter
            textures[i].data = _fp(d)
        mats = (N.MaterialDesc * max(1, len(s.materials)))()
        for i, m in enumerate(s.materials):
            md = mats[i]
            md.type, md.dist, md.two_sided = m.type, m.dist, int(bool(m.two_sided))
            md.tex_r, md.tex_t, md.tex_roughness, md.tex_anisotropic = m.tex_r, m.tex_t, m.tex_roughness, m.tex_anisotropic
            md.eta_a, md.eta_b, md.kd, md.ks = m.eta_a, m.eta_b, m.kd, m.ks
            md.eta[:] = list(m.eta)
            md.k[:] = list(m.k)
        media = (N.MediumDesc * max(1, len(s.media)))()
        for i, m in enumerate(s.media):
            media[i].sigma_a[:] = list(m.sigma_a)
            media[i].sigma_s[:] = list(m.sigma_s)
            media[i].g, media[i].scale = m.g, m.scale

        def pack_group(gd: N.GroupDesc, g: Group):
            gd.kind, gd.ref, gd.material = g.kind, g.ref, g.material
            gd.medium_inside, gd.medium_outside = g.medium_inside, g.medium_outside
            gd.emissive = int(bool(g.emissive))
            gd.le[:] = list(g.le)
            gd.model_to_world[:] = [float(v) for v in g.model_to_world.m]
            if g.kind in (N.GROUP_INSTANCE, N.GROUP_INFINITE_LIGHT):
                gd.world_to_model[:] = [float(v) for v in g.model_to_world.invert().m]
            else:
                gd.world_to_model[:] = [float(v) for v in Mat4.identity().m]

        bgroups = [g for b in s.blas for g in b]
        blas_groups = (N.GroupDesc * max(1, len(bgroups)))()
        for i, g in enumerate(bgroups):
            pack_group(blas_groups[i], g)
        ranges = np.zeros(max(2, 2 * len(s.blas)), dtype=np.int32)
        off = 0
        for i, b in enumerate(s.blas):
            ranges[2 * i], ranges[2 * i + 1] = off, len(b)
            off += len(b)
        keep.append(ranges)
        groups = (N.GroupDesc * max(1, len(s.groups)))()
        for i, g in enumerate(s.groups):
            pack_group(groups[i], g)
        d = N.SceneDescC()
        d.abi_version = N.ABI_VERSION
        d.mesh_count, d.meshes = len(s.meshes), C.cast(meshes, C.POINTER(N.MeshDesc))
        d.sphere_count, d.spheres = len(s.spheres), C.cast(spheres, C.POINTER(N.SphereDesc))
        d.texture_count, d.textures = len(s.textures), C.cast(textures, C.POINTER(N.TextureDesc))
        d.material_count, d.materials = len(s.materials), C.cast(mats, C.POINTER(N.MaterialDesc))
        d.medium_count, d.media = len(s.media), C.cast(media, C.POINTER(N.MediumDesc))
        d.blas_group_count, d.blas_groups = len(bgroups), C.cast(blas_groups, C.POINTER(N.GroupDesc))
        d.blas_count, d.blas_ranges = len(s.blas), ranges.ctypes.data_as(N.IntP)
        d.group_count, d.groups = len(s.groups), C.cast(groups, C.POINTER(N.GroupDesc))
        d.global_medium = s.global_medium
        cam = s.camera
        d.camera.width, d.camera.height = cam.width, cam.height
        d.camera.near_z, d.camera.far_z = cam.near, cam.far
        d.camera.clip_to_camera[:] = [float(v) for v in cam.clip_to_camera().m]
        d.camera.camera_to_world[:] = [float(v) for v in cam.camera_to_world.m]
        d.camera.camera_to_clip[:] = [float(v) for v in cam.camera_to_clip().m]
        d.camera.world_to_camera[:] = [float(v) for v in cam.world_to_camera().m]
        d.bvh_max_prims = s.bvh_max_prims
        self._keep = (keep, meshes, spheres, textures, mats, media, blas_groups, groups)
        self.desc = d
        self.scene = s

    def ref(self):
        return C.byref(self.desc)


# ------------------------------------------------------------- render params ----
@dataclass
class RenderSettings:
    """Integrator + renderer parameters (RendererBuilder.cs:29-72 defaults)."""
    integrator: int = N.INTEGRATOR_PATH
    method: int = N.METHOD_MIS
    strategy: int = N.STRATEGY_UNIFORM
    max_depth: int = -1
    min_depth: int = 3
    rr_threshold: float = 0.99
    spp: int = 256
    seed: int = 1
    sample_begin: int = 0
    x0: int = 0
    y0: int = 0
    width: int = 0
    height: int = 0

    def to_c(self) -> N.RenderParams:
        p = N.RenderParams()
        p.integrator, p.method, p.strategy = self.integrator, self.method, self.strategy
        p.max_depth, p.min_depth, p.rr_threshold = self.max_depth, self.min_depth, self.rr_threshold
        p.spp, p.sample_begin, p.seed = self.spp, self.sample_begin, self.seed
        p.x0, p.y0, p.width, p.height = self.x0, self.y0, self.width, self.height
        return p

    def replace(self, **kw) -> "RenderSettings":
        d = dict(self.__dict__)
        d.update(kw)
        return RenderSettings(**d)
