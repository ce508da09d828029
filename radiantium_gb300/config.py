"""The reference's scene description and plugin registry, host side.

Mirrors Radiantium.Offline/Config: a JSON scene file (the same keys the
reference's CLI reads, Radiantium.Cli/Program.cs:25-142) is fed to a
:class:`RendererBuilder` whose string-keyed registries create integrators,
materials, lights, media, shapes, accelerators and renderers with the
reference's defaults (Config/RendererBuilder.cs:27-234).  ``build()`` walks the
entities like RendererBuilder.Build (RendererBuilder.cs:870-1010) and returns a
:class:`GpuRenderer`, the drop-in replacement of BlockBasedRenderer: the
renderer builders "block_based" and "gpu_wavefront" both create it.

The "adjoint_particle" integrator selects the light tracer
(AdjointParticleRenderer, "particle_count"), rendered by the same class.
Plugins outside the GPU path (octree, bdpt, ao, gbuffer, disney,
subsurface, image files) raise NotImplementedError, the counterpart of the
reference's NotSupportedException.
"""
from __future__ import annotations

import json
import math
import os
import threading
import time

import numpy as np

from . import native as N
from .scene import (Camera, Group, Mat4, Material, Medium, Mesh, RenderSettings, SceneDesc, Sphere, Texture,
                    look_at_left_hand)

F = np.float32

# conductor eta / k in RGB for rough_metal "metal_type" (RGB values of the
# measured spectra pbrt ships; "Cu" is the reference's default)
METALS = {
    "Cu": ((0.1999899, 0.9220823, 1.0998751), (3.9046354, 2.4476316, 2.1376500)),
    "Au": ((0.1428174, 0.3741433, 1.4394432), (3.9747169, 2.3806596, 1.5998082)),
    "Ag": ((0.1549343, 0.1164734, 0.1380863), (4.8180990, 3.1156154, 2.1424003)),
    "Al": ((1.6539409, 0.8784990, 0.5201210), (9.2043056, 6.2562046, 4.8267488)),
}


class ConfigParams:
    """IConfigParamProvider over a parsed JSON object (Config/JsonConfigProvider.cs)."""

    def __init__(self, d=None):
        self.d = d if isinstance(d, dict) else {}

    def has(self, k):
        return k in self.d

    def type_of(self, k):
        v = self.d[k]
        if isinstance(v, bool):
            return "bool"
        if isinstance(v, (int, float)):
            return "number"
        if isinstance(v, str):
            return "string"
        if isinstance(v, list):
            if all(isinstance(x, (int, float)) and not isinstance(x, bool) for x in v):
                return {2: "vec2", 3: "vec3", 4: "vec4", 16: "mat4"}.get(len(v), "array")
            return "array"
        if v is None:
            return "null"
        return "object"

    def int(self, k, default):
        return int(self.d[k]) if k in self.d else default

    def float(self, k, default):
        return float(F(self.d[k])) if k in self.d else default

    def bool(self, k, default):
        return bool(self.d[k]) if k in self.d else default

    def str(self, k, default):
        return str(self.d[k]) if k in self.d else default

    def vec3(self, k, default):
        return tuple(float(F(x)) for x in self.d[k]) if k in self.d else default

    def vec2i(self, k, default):
        return (int(self.d[k][0]), int(self.d[k][1])) if k in self.d else default

    def mat4(self, k, default):
        """ReadMat4: 16 numbers read row-major then transposed."""
        if k not in self.d:
            return default
        v = [F(x) for x in self.d[k]]
        return Mat4([v[(i % 4) * 4 + i // 4] for i in range(16)])

    def sub(self, k):
        return ConfigParams(self.d.get(k))

    def subs(self, k):
        return [ConfigParams(x) for x in self.d.get(k, [])]


def read_transform(p: ConfigParams):
    """RendererBuilderExtension.ReadTransform (RendererBuilder.cs:278-309)."""
    pos = p.vec3("position", (0.0, 0.0, 0.0))
    rot = Mat4.identity()
    if p.has("rotation"):
        t = p.type_of("rotation")
        if t == "mat4":
            rot = p.mat4("rotation", Mat4.identity())
        elif t == "object":
            o = p.sub("rotation")
            axis = o.vec3("axis", (0.0, 1.0, 0.0))
            angle = o.float("angle", 0.0)
            rot = Mat4.from_axis_angle(axis, float(F(angle) * (F(3.14159265) / F(180))))
        elif t == "vec4":
            x, y, z, w = (F(v) for v in p.d["rotation"])
            rot = _from_quaternion(x, y, z, w)
        else:
            raise ValueError("invalid rotation param")
    scale = p.vec3("scale", (1.0, 1.0, 1.0))
    return pos, rot, scale


def _from_quaternion(x, y, z, w):
    """Matrix4x4.CreateFromQuaternion: rotation matrix of a unit quaternion (row vectors)."""
    xx, yy, zz = x * x, y * y, z * z
    xy, wz, xz, wy, yz, wx = x * y, z * w, z * x, y * w, y * z, x * w
    one, two = F(1), F(2)
    return Mat4([one - two * (yy + zz), two * (xy + wz), two * (xz - wy), 0,
                 two * (xy - wz), one - two * (zz + xx), two * (yz + wx), 0,
                 two * (xz + wy), two * (yz - wx), one - two * (yy + xx), 0,
                 0, 0, 0, 1])


def read_obj(path: str, will_gen_normal: bool = False) -> Mesh:
    """Triangle OBJ reader: v / vt / vn / f with (position, normal, texcoord) vertex
    de-duplication in face order (Radiantium.Core/WavefrontObjReader.cs:445-501)."""
    pos, nrm, tex, faces = [], [], [], []
    with open(path) as f:
        for line in f:
            if line.startswith("v "):
                pos.append([float(v) for v in line.split()[1:4]])
            elif line.startswith("vn "):
                nrm.append([float(v) for v in line.split()[1:4]])
            elif line.startswith("vt "):
                tex.append([float(v) for v in line.split()[1:3]])
            elif line.startswith("f "):
                vs = line.split()[1:]
                if len(vs) != 3:
                    raise ValueError(f"{path}: only triangle faces are supported")
                tri = []
                for v in vs:
                    parts = (v.split("/") + ["", ""])[:3]
                    tri.append(tuple(int(x) - 1 if x else -1 for x in parts))
                faces.append(tri)
    unique, p, n, u, ind = {}, [], [], [], []
    for tri in faces:
        for (vi, ti, ni) in tri:
            key = (vi, ni, ti)
            idx = unique.get(key)
            if idx is None:
                idx = len(p)
                unique[key] = idx
                p.append(pos[vi])
                if ni >= 0:
                    n.append(nrm[ni])
                elif will_gen_normal:
                    n.append([0.0, 0.0, 0.0])
                if ti >= 0:
                    u.append(tex[ti])
            ind.append(idx)
    P = np.asarray(p, dtype=np.float32)
    I = np.asarray(ind, dtype=np.int32).reshape(-1, 3)
    Nn = np.asarray(n, dtype=np.float32) if n else None
    if will_gen_normal and not nrm:
        for t in I:
            a, b, c = P[t[0]], P[t[1]], P[t[2]]
            cr = np.cross(b - a, c - a).astype(np.float32)
            nor = cr / np.float32(np.sqrt(np.float32(np.dot(cr, cr))))
            na = Nn[t[0]].copy()   # the reference reads the first corner's normal for all three
            for k in range(3):
                Nn[t[k]] = nor if not na.any() else (nor + na) / np.linalg.norm(nor + na)
    U = np.asarray(u, dtype=np.float32) if u else None
    return Mesh(P, I, Nn, U)


class GpuRenderer:
    """Renderer (Radiantium.Offline/Renderer.cs) rendering on one GPU through the C ABI.

    Samples are rendered in progressive passes so that Stop() and the task
    counters behave like BlockBasedRenderer's blocks."""

    def __init__(self, scene: SceneDesc, settings: RenderSettings, device: int = 0, passes: int = 0,
                 particle_count: int = 0, traversal: int = N.TRAVERSAL_EXACT,
                 light_sampling: int = N.LIGHT_SAMPLING_CDF):
        self.scene, self.settings, self.device = scene, settings, device
        self.particle_count = particle_count
        self.traversal, self.light_sampling = traversal, light_sampling
        work = particle_count if settings.integrator == N.INTEGRATOR_PARTICLE else settings.spp
        self.passes = passes or min(work, 16)
        self._target = np.zeros((scene.camera.width, scene.camera.height, 3), dtype=np.float32)
        self._thread = None
        self._done = 0
        self._error = None
        self._stop = threading.Event()
        self._t0 = self._t1 = None
        self._dev = None

    # -- Renderer contract ----------------------------------------------------
    @property
    def RenderTarget(self):
        return self._target

    @property
    def IsCompleted(self):
        return self._thread is not None and not self._thread.is_alive()

    @property
    def IsSuccess(self):
        return self._error is None

    @property
    def AllTaskCount(self):
        return self.passes

    @property
    def CompletedTaskCount(self):
        return self._done

    @property
    def ElapsedTime(self):
        if self._t0 is None:
            return 0.0
        return (self._t1 or time.perf_counter()) - self._t0

    def Start(self):
        if self._thread is None:
            self._t0 = time.perf_counter()
            self._thread = threading.Thread(target=self._run, daemon=True)
            self._thread.start()
        return self._thread

    def Wait(self):
        if self._thread is None:
            raise RuntimeError("no render task start")
        self._thread.join()
        if self._error is not None:
            raise self._error

    def Stop(self):
        self._stop.set()
        if self._dev is not None:
            self._dev.cancel()

    def _run(self):
        from .device import Device
        try:
            with Device(self.device) as dev:
                self._dev = dev
                dev.set_traversal(self.traversal)
                dev.set_light_sampling(self.light_sampling)
                dev.upload(self.scene)
                st = self.settings
                acc = np.zeros_like(self._target, dtype=np.float64)
                if st.integrator == N.INTEGRATOR_PARTICLE:
                    self._run_particles(dev, acc)
                    self._dev = None
                    return
                done_spp = 0
                per = [st.spp // self.passes + (1 if i < st.spp % self.passes else 0) for i in range(self.passes)]
                for k in per:
                    if self._stop.is_set() or k == 0:
                        break
                    img = dev.render(st.replace(spp=k, sample_begin=st.sample_begin + done_spp))
                    acc += img.astype(np.float64) * k
                    done_spp += k
                    self._done += 1
                    self._target[...] = (acc / done_spp).astype(np.float32)
                self._dev = None
        except Exception as e:  # reported through IsSuccess / Wait like the reference's _hasException
            self._error = e
        finally:
            self._t1 = time.perf_counter()

    def _run_particles(self, dev, acc):
        """AdjointParticleRenderer: particle ranges per pass; a film of n particles
        weighs n / N in the running mean (each film is already scaled by 1/n)."""
        n_all, done = self.particle_count, 0
        per = [n_all // self.passes + (1 if i < n_all % self.passes else 0) for i in range(self.passes)]
        for k in per:
            if self._stop.is_set() or k == 0:
                break
            img = dev.render_particles(self.settings, k, first=done)
            acc += img.astype(np.float64) * k
            done += k
            self._done += 1
            self._target[...] = (acc / done).astype(np.float32)


def gpu_modes(rc: ConfigParams) -> dict:
    """The GPU renderer's own options in the "renderer" object (no reference
    counterpart; the reference ignores keys it does not read): "traversal"
    "exact" (default) or "wide", "light_sampling" "cdf" (default) or "alias"."""
    trav = {"exact": N.TRAVERSAL_EXACT, "wide": N.TRAVERSAL_WIDE}
    ls = {"cdf": N.LIGHT_SAMPLING_CDF, "alias": N.LIGHT_SAMPLING_ALIAS}
    t, l = rc.str("traversal", "exact"), rc.str("light_sampling", "cdf")
    if t not in trav:
        raise ValueError(f"renderer.traversal: {t!r} is not one of {sorted(trav)}")
    if l not in ls:
        raise ValueError(f"renderer.light_sampling: {l!r} is not one of {sorted(ls)}")
    return {"traversal": trav[t], "light_sampling": ls[l]}


class RendererBuilder:
    """Config/RendererBuilder.cs: registries + entity graph -> GpuRenderer."""

    def __init__(self, search_path: str = ".", workspace: str = "scene"):
        self.search_path, self.workspace = search_path, workspace
        self.integrators, self.materials, self.area_lights, self.infinite_lights = {}, {}, {}, {}
        self.media, self.shapes, self.accels, self.renderers = {}, {}, {}, {}
        self.models, self.images, self.instanced, self.entities, self.roots = {}, {}, [], [], []
        self.renderer_cfg = self.integrator_cfg = self.camera_cfg = self.accel_cfg = None
        self.global_medium_cfg = None
        self.scene: SceneDesc | None = None

    # -- registration (AddXxxBuilder) -------------------------------------------------------------
    def set_default_builders(self):
        """RendererBuilderExtension.SetDefaultBuilders, restricted to the GPU path's plugins."""
        def path(b, p):
            meth = {"Bxdf": N.METHOD_BXDF, "Nee": N.METHOD_NEE, "Mis": N.METHOD_MIS}[p.str("method", "Mis")]
            strat = {"Uniform": N.STRATEGY_UNIFORM, "All": N.STRATEGY_ALL}[p.str("strategy", "Uniform")]
            return RenderSettings(N.INTEGRATOR_PATH, meth, strat, p.int("max_depth", -1), p.int("min_depth", 3),
                                  p.float("rr_threshold", 0.99))

        def vol_path(b, p):
            strat = {"Uniform": N.STRATEGY_UNIFORM, "All": N.STRATEGY_ALL}[p.str("strategy", "Uniform")]
            return RenderSettings(N.INTEGRATOR_VOL_PATH, N.METHOD_MIS, strat, p.int("max_depth", -1),
                                  p.int("min_depth", 3), p.float("rr_threshold", 0.99))

        def adjoint_particle(b, p):
            return RenderSettings(N.INTEGRATOR_PARTICLE, N.METHOD_MIS, N.STRATEGY_UNIFORM, p.int("max_depth", -1),
                                  p.int("min_depth", 3), p.float("rr_threshold", 0.99))

        self.integrators.update({"path": path, "vol_path": vol_path, "adjoint_particle": adjoint_particle})
        self.accels["bvh"] = lambda b, p: max(1, p.int("max_prim", 1))

        def dist(p, default):
            return {"Beckmann": N.DIST_BECKMANN, "GGX": N.DIST_GGX}[p.str("dist", default)]

        def diffuse(b, p):
            return Material(N.MAT_DIFFUSE, tex_r=b.tex(p, "kd", 0.5), two_sided=p.bool("is_two_side", False))

        def perfect_glass(b, p):
            return Material(N.MAT_PERFECT_GLASS, tex_r=b.tex(p, "r", 1.0), tex_t=b.tex(p, "t", 1.0),
                            eta_a=p.float("etaA", 1.000277), eta_b=p.float("etaB", 1.5046))

        def perfect_mirror(b, p):
            return Material(N.MAT_PERFECT_MIRROR, tex_r=b.tex(p, "r", 1.0), two_sided=p.bool("is_two_side", False))

        def rough_plastic(b, p):
            return Material(N.MAT_ROUGH_PLASTIC, dist(p, "Beckmann"), p.bool("is_two_side", False),
                            tex_r=b.tex(p, "r", 0.5), tex_roughness=b.tex(p, "roughness", 0.3),
                            tex_anisotropic=b.tex(p, "anisotropic", 0.0), kd=p.float("kd", 0.5), ks=p.float("ks", 0.5),
                            eta_a=p.float("etaA", 1.000277), eta_b=p.float("etaB", 1.5046))

        def rough_metal(b, p):
            eta, k = METALS["Cu"]
            if p.has("metal_type"):
                if p.type_of("metal_type") == "string":
                    name = p.str("metal_type", "Cu")
                    if name not in METALS:
                        raise NotImplementedError(f"metal type {name} is not in the host table")
                    eta, k = METALS[name]
                else:
                    eta, k = p.vec3("eta", eta), p.vec3("k", k)
            return Material(N.MAT_ROUGH_METAL, dist(p, "GGX"), p.bool("is_two_side", False),
                            tex_roughness=b.tex(p, "roughness", 0.3), tex_anisotropic=b.tex(p, "anisotropic", 0.0),
                            eta=eta, k=k)

        def rough_glass(b, p):
            return Material(N.MAT_ROUGH_GLASS, dist(p, "GGX"), tex_r=b.tex(p, "r", 1.0), tex_t=b.tex(p, "t", 1.0),
                            tex_roughness=b.tex(p, "roughness", 0.3), tex_anisotropic=b.tex(p, "anisotropic", 0.0),
                            eta_a=p.float("etaA", 1.000277), eta_b=p.float("etaB", 1.5046))

        self.materials.update({"diffuse": diffuse, "perfect_glass": perfect_glass, "perfect_mirror": perfect_mirror,
                               "rough_plastic": rough_plastic, "rough_metal": rough_metal, "rough_glass": rough_glass})
        self.area_lights["diffuse_area"] = lambda b, p: p.vec3("le", (1.0, 1.0, 1.0))
        self.infinite_lights["infinite"] = lambda b, p: b.tex(p, "le", 0.0)
        self.media["homogeneous"] = lambda b, p: Medium(p.vec3("sigma_a", (0.0, 0.0, 0.0)),
                                                        p.vec3("sigma_s", (0.0, 0.0, 0.0)), p.float("g", 0.0),
                                                        p.float("scale", 1.0))
        self.shapes["sphere"] = lambda b, m, p: (p.vec3("center", (0.0, 0.0, 0.0)), p.float("radius", 0.5), m)
        for name in ("block_based", "gpu_wavefront"):
            self.renderers[name] = lambda b, p: (p.int("spp", 256), p.int("block_size", 32), p.int("threads", -1))
        self.renderers["adjoint_particle"] = lambda b, p: (p.int("particle_count", 16384), p.int("threads", -1))
        return self

    # -- texture parameter (RendererBuilderExtension.ReadTex2D) ------------------------------------
    def tex(self, p: ConfigParams, key: str, default) -> int:
        s = self.scene
        if not p.has(key):
            return s.add_const(default)
        t = p.type_of(key)
        if t == "vec3":
            return s.add_const(p.vec3(key, (0, 0, 0)))
        if t == "number":
            return s.add_const(p.float(key, 0.0))
        cfg = p.sub(key)
        if cfg.str("type", "") == "image":
            name = cfg.str("name", None)
            if name not in self.images:
                raise NotImplementedError(f"image texture {name}: only images provided as arrays are supported")
            smp = cfg.sub("sampler")
            wrap = {"Clamp": N.WRAP_CLAMP, "Repeat": N.WRAP_REPEAT}[smp.str("wrap", "Clamp")]
            filt = {"Nearest": N.FILTER_NEAREST, "Linear": N.FILTER_LINEAR}[smp.str("filter", "Nearest")]
            img = self.images[name]
            return s.add_texture(Texture.from_image_hw3(img, wrap, filt))
        raise NotImplementedError(f"texture type {cfg.str('type', '?')}")

    def add_image(self, name: str, img_hw3: np.ndarray):
        """Registers an already decoded image (h, w, 3 float) under an asset name."""
        self.images[name] = np.asarray(img_hw3, dtype=np.float32)

    # -- configuration (SetXxx / AddXxx) -----------------------------------------------------------
    def load(self, cfg: ConfigParams):
        """Radiantium.Cli/Program.cs:GetRenderer: reads one parsed scene file."""
        if cfg.has("renderer"):
            self.renderer_cfg = cfg.sub("renderer")
        if cfg.has("integrator"):
            self.integrator_cfg = cfg.sub("integrator")
        self.camera_cfg = cfg.sub("camera")
        if self.camera_cfg.has("medium"):
            self.global_medium_cfg = self.camera_cfg.sub("medium")
        if cfg.has("accel"):
            self.accel_cfg = cfg.sub("accel")
        self.output_cfg = cfg.sub("output") if cfg.has("output") else None
        for a in cfg.subs("assets"):
            t = a.str("type", None)
            if t == "model":
                loc = self._path(a.str("location", ""))
                self.models[a.str("name", "")] = read_obj(loc, a.bool("will_gen_normal", False))
            elif t == "image":
                if a.str("name", "") not in self.images:
                    raise NotImplementedError("image assets must be added with add_image() (no image decoder)")
            else:
                raise ValueError(f"unknown asset type {t}")
        for ins in cfg.subs("instanced"):
            self.instanced.append(ins)
        q = [(e, None) for e in cfg.subs("scene")]
        while q:
            e, parent = q.pop(0)
            idx = len(self.entities)
            self.entities.append({"cfg": e, "parent": parent, "children": []})
            if parent is None:
                self.roots.append(idx)
            else:
                self.entities[parent]["children"].append(idx)
            q.extend((c, idx) for c in e.subs("children"))
        return self

    def _path(self, loc):
        if os.path.exists(loc):
            return loc
        p = os.path.normpath(os.path.join(self.search_path, loc))
        if not os.path.exists(p):
            raise FileNotFoundError(f"invalid location {loc}")
        return p

    @staticmethod
    def _local(p: ConfigParams):
        pos, rot, scale = read_transform(p.sub("transform")) if p.has("transform") else ((0, 0, 0), Mat4.identity(), (1, 1, 1))
        return Mat4.scale(scale) * rot * Mat4.translation(pos)

    def _camera(self) -> Camera:
        p = self.camera_cfg
        if p.str("type", None) != "perspective":
            raise NotImplementedError(f"camera {p.str('type', None)}")
        w, h = p.vec2i("screen", (1280, 720))
        fov, near, far = p.float("fov", 60.0), p.float("near", 0.001), p.float("far", 1000.0)
        if p.has("origin"):
            m = look_at_left_hand(p.vec3("origin", (0, 0, 3)), p.vec3("target", (0, 0, 0)), p.vec3("up", (0, 1, 0)))
        else:
            m = p.mat4("to_world", Mat4.identity())
        return Camera(w, h, fov, near, far, m)

    def _medium(self, p: ConfigParams | None) -> int:
        if p is None or not p.d:
            return -1
        if p.bool("is_global", False):
            return self.scene.global_medium
        t = p.str("type", None)
        if t not in self.media:
            raise NotImplementedError(f"medium {t}")
        return self.scene.add_medium(self.media[t](self, p))

    def _medium_adapter(self, p: ConfigParams | None):
        if p is None or not p.d:
            return -1, -1
        if p.has("same"):
            m = self._medium(p.sub("same"))
            return m, m
        outside = self._medium(p.sub("outside")) if p.has("outside") else -1
        inside = self._medium(p.sub("inside")) if p.has("inside") else -1
        return inside, outside

    def _shape_groups(self, shapes, models, m2w: Mat4, **g):
        out = []
        for sp in shapes:
            t = sp.str("type", None)
            if t not in self.shapes:
                raise NotImplementedError(f"shape {t}")
            c, r, mat = self.shapes[t](self, m2w, sp)
            from .scene import transform_points
            center = transform_points(np.array([c], dtype=np.float32), mat)[0]
            self.scene.spheres.append(Sphere(tuple(float(v) for v in center), r, mat))
            out.append(Group(N.GROUP_SPHERE, len(self.scene.spheres) - 1, **g))
        for mp in models:
            name = mp.str("name", None)
            if mp.has("child"):
                raise NotImplementedError("OBJ sub-models")
            mesh = self.models[name].transformed(m2w)
            out.append(Group(N.GROUP_MESH, self.scene.add_mesh(mesh), **g))
        return out

    def build(self, device: int = 0) -> GpuRenderer:
        """RendererBuilder.Build (RendererBuilder.cs:870-1010)."""
        s = self.scene = SceneDesc(camera=self._camera(), name=self.workspace)
        if self.accel_cfg is not None:
            t = self.accel_cfg.str("type", None)
            if t not in self.accels:
                raise NotImplementedError(f"accelerator {t}")
            s.bvh_max_prims = self.accels[t](self, self.accel_cfg)
        # instanced prototypes
        for ins in self.instanced:
            if ins.has("accel") and ins.sub("accel").str("type", "bvh") != "bvh":
                raise NotImplementedError("instanced accelerators other than bvh")
            m = self._local(ins)
            shp = ins.sub("shape")
            shapes = [shp] if shp.d and shp.str("type", None) != "model" else []
            models = [shp] if shp.d and shp.str("type", None) == "model" else []
            s.blas.append(self._shape_groups(shapes, models, m))
        s.global_medium = self._medium(self.global_medium_cfg) if self.global_medium_cfg else -1
        # entity transforms, breadth first
        order = list(self.roots)
        m2w = {}
        while order:
            i = order.pop(0)
            e = self.entities[i]
            par = m2w[e["parent"]] if e["parent"] is not None else Mat4.identity()
            m2w[i] = par * self._local(e["cfg"])
            order.extend(e["children"])
        for i, e in enumerate(self.entities):
            c = e["cfg"]
            mat_cfg = c.sub("material") if c.has("material") else None
            med_cfg = c.sub("medium") if c.has("medium") else None
            light_cfg = c.sub("light") if c.has("light") else None
            if mat_cfg is None and med_cfg is None:
                if light_cfg is None:
                    continue
                t = light_cfg.str("type", None)
                if t not in self.infinite_lights:
                    raise NotImplementedError(f"infinite light {t}")
                s.groups.append(Group(N.GROUP_INFINITE_LIGHT, self.infinite_lights[t](self, light_cfg),
                                      model_to_world=m2w[i]))
                continue
            mat = -1
            if mat_cfg is not None:
                t = mat_cfg.str("type", None)
                if t not in self.materials:
                    raise NotImplementedError(f"material {t}")
                mat = s.add_material(self.materials[t](self, mat_cfg))
            inside, outside = self._medium_adapter(med_cfg)
            le, emissive = (0.0, 0.0, 0.0), False
            if light_cfg is not None:
                t = light_cfg.str("type", None)
                if t not in self.area_lights:
                    raise NotImplementedError(f"area light {t}")
                le, emissive = self.area_lights[t](self, light_cfg), True
            g = dict(material=mat, medium_inside=inside, medium_outside=outside, emissive=emissive, le=le)
            shp = c.sub("shape") if c.has("shape") else ConfigParams()
            shapes = [shp] if shp.d and shp.str("type", None) != "model" else []
            models = [shp] if shp.d and shp.str("type", None) == "model" else []
            s.groups.extend(self._shape_groups(shapes, models, m2w[i], **g))
            if c.has("instanced"):
                s.groups.append(Group(N.GROUP_INSTANCE, c.sub("instanced").int("id", -1), material=mat,
                                      medium_inside=inside, medium_outside=outside, model_to_world=m2w[i]))
        # integrator + renderer
        ic = self.integrator_cfg
        if ic is None or ic.str("type", None) not in self.integrators:
            raise NotImplementedError(f"integrator {None if ic is None else ic.str('type', None)}")
        settings = self.integrators[ic.str("type", None)](self, ic)
        rc = self.renderer_cfg if self.renderer_cfg is not None else ConfigParams()
        modes = gpu_modes(rc)
        if settings.integrator == N.INTEGRATOR_PARTICLE:
            # the renderer named by the integrator (AdjointParticleIntegrator.cs:15, RendererBuilder.cs:523)
            return GpuRenderer(s, settings, device, particle_count=self.renderers["adjoint_particle"](self, rc)[0],
                               **modes)
        settings = settings.replace(spp=self.renderers["block_based"](self, rc)[0])
        return GpuRenderer(s, settings, device, **modes)


def load_scene_file(path: str, device: int = 0) -> GpuRenderer:
    """Equivalent of the reference CLI's GetRenderer for one JSON scene file."""
    return load_scene_file_with_output(path, device)[0]


def load_scene_file_with_output(path: str, device: int = 0):
    """GetRenderer (Radiantium.Cli/Program.cs:25-142) with its ResultOutput:
    (renderer, output); after Wait(), output.save(renderer) writes the files."""
    from .output import ResultOutput
    with open(path) as f:
        cfg = ConfigParams(json.load(f))
    b = RendererBuilder(os.path.dirname(os.path.abspath(path)),
                        os.path.splitext(os.path.basename(path))[0]).set_default_builders()
    b.load(cfg)
    out = ResultOutput.from_config(getattr(b, "output_cfg", None), b.search_path, b.workspace)
    return b.build(device), out
