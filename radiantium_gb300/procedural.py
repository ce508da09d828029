"""Seeded procedural scenes for the benchmark workloads.

The reference ships no benchmark scenes; these generators build, from a seed,
the workloads its headline metric is quoted on:

* :func:`cornell_box`  - plain path integrator, procedural Cornell box in a unit
  cube: 5 wall quads (10 tris), 2 rotated boxes (24 tris), a ceiling quad light
  (radiance 15), Lambertian albedos 0.73 / 0.65 / 0.12, 256x256, 64 spp, depth 5.
* :func:`instanced_spheres` - 64 instances of a ~200k-triangle displaced sphere,
  GGX conductors (alpha ~ U[0.05, 0.5]) and rough dielectrics (IOR 1.5), lit
  by a 1024x512 HDR environment of 8 Gaussian lobes, 1024x1024, 256 spp, depth 8.
* :func:`volume_sphere` - vol_path: ~500k-triangle displaced sphere bounding a
  homogeneous medium (sigma_a 0.05, sigma_s 2.0, HG g 0.7) over a diffuse
  ground with one quad light, 512x512, 512 spp, depth 32.

Every scene is a :class:`~radiantium_gb300.scene.SceneDesc` built through the
same tables the reference's RendererBuilder fills (meshes per entity,
materials with texture parameters, instanced prototypes, infinite light).
Only IEEE-exact float operations (and float64 noise rounded to float32) are
used so the meshes are identical on x86-64 and aarch64.
"""
from __future__ import annotations

import math

import numpy as np

from . import native as N
from .scene import (Camera, Group, Mat4, Material, Medium, Mesh, RenderSettings, SceneDesc, Texture,
                    transform_points)

# copper conductor eta / k in RGB (rough_metal default metal_type "Cu")
CU_ETA = (0.1999899, 0.9220823, 1.0998751)
CU_K = (3.9046354, 2.4476316, 2.1376500)


# ------------------------------------------------------------------ geometry ----
def quad(p0, p1, p2, p3) -> Mesh:
    """Two triangles (p0,p1,p2), (p0,p2,p3); normal = normalize(cross(p1-p0, p2-p0))."""
    pos = np.array([p0, p1, p2, p3], dtype=np.float32)
    return Mesh(pos, np.array([[0, 1, 2], [0, 2, 3]], dtype=np.int32))


def box_mesh(center, size, angle_deg) -> Mesh:
    """Axis-aligned box of `size`, rotated about +y by `angle_deg`, outward normals."""
    sx, sy, sz = (s * 0.5 for s in size)
    corners = np.array([[x, y, z] for x in (-sx, sx) for y in (-sy, sy) for z in (-sz, sz)], dtype=np.float64)
    a = math.radians(angle_deg)
    c, s = math.cos(a), math.sin(a)
    rot = np.array([[c, 0, -s], [0, 1, 0], [s, 0, c]])
    pts = (corners @ rot.T + np.asarray(center)).astype(np.float32)
    # faces as corner index quads (x,y,z bits: x*4 + y*2 + z)
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    idx = []
    for q in faces:
        idx += [[q[0], q[1], q[2]], [q[0], q[2], q[3]]]
    idx = np.array(idx, dtype=np.int32)
    idx = _orient_outward(pts, idx, pts.mean(axis=0))
    return Mesh(pts, idx)


def _orient_outward(pos, idx, center):
    a, b, c = pos[idx[:, 0]].astype(np.float64), pos[idx[:, 1]].astype(np.float64), pos[idx[:, 2]].astype(np.float64)
    n = np.cross(b - a, c - a)
    out = ((a + b + c) / 3.0) - np.asarray(center, dtype=np.float64)
    flip = (n * out).sum(axis=1) < 0
    idx = idx.copy()
    idx[flip] = idx[flip][:, [0, 2, 1]]
    return idx


def _hash3(ix, iy, iz, seed):
    """Integer lattice hash (xorshift-multiply mix) -> float64 in [-1, 1)."""
    h = (ix.astype(np.uint64) * np.uint64(0x8DA6B343) ^ iy.astype(np.uint64) * np.uint64(0xD8163841)
         ^ iz.astype(np.uint64) * np.uint64(0xCB1AB31F) ^ np.uint64(seed) * np.uint64(0x9E3779B97F4A7C15))
    h = h & np.uint64(0xFFFFFFFFFFFFFFFF)
    h ^= h >> np.uint64(33)
    h *= np.uint64(0xFF51AFD7ED558CCD)
    h ^= h >> np.uint64(33)
    h *= np.uint64(0xC4CEB9FE1A85EC53)
    h ^= h >> np.uint64(33)
    return (h >> np.uint64(11)).astype(np.float64) * (2.0 / 9007199254740992.0) - 1.0


def value_noise(p: np.ndarray, seed: int, octaves: int = 3) -> np.ndarray:
    """Seeded 3-D value noise (smoothstep-interpolated lattice values), fBm sum in [-1, 1]."""
    total = np.zeros(p.shape[0])
    amp, norm, freq = 1.0, 0.0, 1.0
    with np.errstate(over="ignore"):
        for o in range(octaves):
            q = p * freq
            i0 = np.floor(q)
            f = q - i0
            w = f * f * (3.0 - 2.0 * f)
            i0 = i0.astype(np.int64) + 1024
            acc = np.zeros(p.shape[0])
            for dx in (0, 1):
                for dy in (0, 1):
                    for dz in (0, 1):
                        val = _hash3(i0[:, 0] + dx, i0[:, 1] + dy, i0[:, 2] + dz, seed * 131 + o)
                        wx = w[:, 0] if dx else 1.0 - w[:, 0]
                        wy = w[:, 1] if dy else 1.0 - w[:, 1]
                        wz = w[:, 2] if dz else 1.0 - w[:, 2]
                        acc += val * wx * wy * wz
            total += amp * acc
            norm += amp
            amp *= 0.5
            freq *= 2.0
    return total / norm


def displaced_sphere(n: int, seed: int, amplitude: float = 0.06, frequency: float = 3.0) -> Mesh:
    """Cube-sphere with n x n quads per face (12 n^2 triangles), radius 1 + amplitude * noise,
    counter-clockwise seen from outside.  Seam vertices are computed from identical
    cube coordinates, so shared edges have bit-identical end points."""
    t = np.tan((np.arange(n + 1) / n * 2.0 - 1.0) * (math.pi / 4.0))  # equal-angle warp
    u, v = np.meshgrid(t, t, indexing="ij")
    u, v = u.reshape(-1), v.reshape(-1)
    one = np.ones_like(u)
    faces = [np.stack([one, u, v], 1), np.stack([-one, v, u], 1), np.stack([v, one, u], 1),
             np.stack([u, -one, v], 1), np.stack([u, v, one], 1), np.stack([v, u, -one], 1)]
    pos, idx = [], []
    g = np.arange((n + 1) * (n + 1)).reshape(n + 1, n + 1)
    a, b, c, d = g[:-1, :-1].reshape(-1), g[1:, :-1].reshape(-1), g[1:, 1:].reshape(-1), g[:-1, 1:].reshape(-1)
    quad_idx = np.concatenate([np.stack([a, b, c], 1), np.stack([a, c, d], 1)])
    for k, f in enumerate(faces):
        pos.append(f)
        idx.append(quad_idx + k * (n + 1) * (n + 1))
    cube = np.concatenate(pos)
    idx = np.concatenate(idx).astype(np.int32)
    dirs = cube / np.sqrt((cube * cube).sum(1, keepdims=True))
    # amplitude 0 (the displaced box's base sphere) leaves r = 1 exactly: skip the noise
    r = 1.0 + amplitude * value_noise(dirs * frequency, seed) if amplitude != 0.0 else np.ones(dirs.shape[0])
    p = (dirs * r[:, None]).astype(np.float32)
    idx = _orient_outward(p, idx, np.zeros(3))
    return Mesh(p, idx)


def gaussian_lobe_env(width: int, height: int, seed: int, lobes: int = 8) -> Texture:
    """Lat-long HDR radiance map: sky base + `lobes` Gaussian lobes on the sphere.
    Texel (x, y) covers phi = 2 pi (x+0.5)/w, theta = pi (y+0.5)/h with the
    direction convention of InfiniteAreaLight.Le (phi = atan2(x, -z), theta = acos y)."""
    rng = np.random.default_rng(seed)
    phi = (np.arange(width) + 0.5) / width * 2 * math.pi
    theta = (np.arange(height) + 0.5) / height * math.pi
    th, ph = np.meshgrid(theta, phi, indexing="ij")  # (h, w)
    d = np.stack([np.sin(th) * np.sin(ph), np.cos(th), -np.sin(th) * np.cos(ph)], -1)
    img = np.zeros((height, width, 3)) + np.array([0.03, 0.04, 0.06]) * (0.5 + 0.5 * d[..., 1:2].clip(0, 1))
    for k in range(lobes):
        z = rng.uniform(-0.2, 1.0)
        a = rng.uniform(0, 2 * math.pi)
        axis = np.array([math.sqrt(1 - z * z) * math.cos(a), z, math.sqrt(1 - z * z) * math.sin(a)])
        sharp = rng.uniform(8.0, 400.0) if k else 2000.0
        color = rng.uniform(0.2, 1.0, 3) * (rng.uniform(2.0, 20.0) if k else 200.0)
        img += color * np.exp((d @ axis - 1.0) * sharp)[..., None]
    return Texture.from_image_hw3(img.astype(np.float32))


# -------------------------------------------------------------------- scenes ----
def cornell_box(width=256, height=256):
    """Procedural Cornell box in the unit cube [0,1]^3, open towards +z."""
    s = SceneDesc(camera=Camera.look_at(width, height, 40.0, (0.5, 0.5, 2.3), (0.5, 0.5, 0.0)), name="cornell")
    white = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const((0.73, 0.73, 0.73))))
    red = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const((0.65, 0.05, 0.05))))
    green = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const((0.12, 0.45, 0.15))))
    lightmat = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const((0.5, 0.5, 0.5))))
    # inward-facing walls: floor, ceiling, back, left (red), right (green)
    walls = [
        (quad((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0)), white),
        (quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)), white),
        (quad((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)), white),
        (quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)), red),
        (quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0)), green),
    ]
    for mesh, m in walls:
        s.groups.append(Group(N.GROUP_MESH, s.add_mesh(mesh), material=m))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(box_mesh((0.66, 0.15, 0.62), (0.3, 0.3, 0.3), -17.0)), material=white))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(box_mesh((0.34, 0.3, 0.36), (0.3, 0.6, 0.3), 17.0)), material=white))
    light = quad((0.4, 0.999, 0.4), (0.6, 0.999, 0.4), (0.6, 0.999, 0.6), (0.4, 0.999, 0.6))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(light), material=lightmat, emissive=True, le=(15.0, 15.0, 15.0)))
    settings = RenderSettings(N.INTEGRATOR_PATH, N.METHOD_MIS, N.STRATEGY_UNIFORM, max_depth=5, min_depth=3,
                              rr_threshold=0.99, spp=64, seed=1)
    return s, settings


def instanced_spheres(width=1024, height=1024, sphere_n=129, grid=8, env_w=1024, env_h=512, seed=7):
    """64 instances of one displaced sphere (12 * 129^2 = 199,692 triangles)."""
    rng = np.random.default_rng(seed)
    s = SceneDesc(camera=Camera.look_at(width, height, 40.0, (0.0, 13.0, 21.0), (0.0, 0.0, 0.0)), name="instanced")
    proto = s.add_mesh(displaced_sphere(sphere_n, seed))
    s.blas.append([Group(N.GROUP_MESH, proto)])
    zero = s.add_const(0.0)
    one = s.add_const(1.0)
    spacing = 2.6
    for gi in range(grid):
        for gj in range(grid):
            alpha = float(rng.uniform(0.05, 0.5))
            rough = s.add_const(math.sqrt(alpha))
            if (gi + gj) % 2 == 0:
                m = s.add_material(Material(N.MAT_ROUGH_METAL, N.DIST_GGX, tex_roughness=rough, tex_anisotropic=zero,
                                            eta=CU_ETA, k=CU_K))
            else:
                m = s.add_material(Material(N.MAT_ROUGH_GLASS, N.DIST_GGX, tex_r=one, tex_t=one, tex_roughness=rough,
                                            tex_anisotropic=zero, eta_a=1.0, eta_b=1.5))
            scale = float(rng.uniform(1.0, 1.25))
            ang = float(rng.uniform(0, 2 * math.pi))
            pos = ((gi - (grid - 1) / 2) * spacing, scale, (gj - (grid - 1) / 2) * spacing)
            m2w = Mat4.scale((scale, scale, scale)) * Mat4.from_axis_angle((0, 1, 0), ang) * Mat4.translation(pos)
            s.groups.append(Group(N.GROUP_INSTANCE, 0, material=m, model_to_world=m2w))
    env = s.add_texture(gaussian_lobe_env(env_w, env_h, seed))
    s.groups.append(Group(N.GROUP_INFINITE_LIGHT, env))
    settings = RenderSettings(N.INTEGRATOR_PATH, N.METHOD_MIS, N.STRATEGY_UNIFORM, max_depth=8, min_depth=3,
                              rr_threshold=0.99, spp=256, seed=1)
    return s, settings


def volume_sphere(width=512, height=512, sphere_n=204, seed=11):
    """vol_path: displaced sphere (12 * 204^2 = 499,392 triangles) with no material
    bounding a homogeneous medium, diffuse ground, one quad light."""
    s = SceneDesc(camera=Camera.look_at(width, height, 45.0, (0.0, 1.6, 5.0), (0.0, 1.0, 0.0)), name="volume")
    ground = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const((0.5, 0.5, 0.5))))
    lightmat = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const((0.5, 0.5, 0.5))))
    med = s.add_medium(Medium((0.05, 0.05, 0.05), (2.0, 2.0, 2.0), g=0.7, scale=1.0))
    sph = displaced_sphere(sphere_n, seed, amplitude=0.08).transformed(Mat4.translation((0.0, 1.1, 0.0)))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(sph), material=-1, medium_inside=med, medium_outside=-1))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(quad((-10, 0, -10), (-10, 0, 10), (10, 0, 10), (10, 0, -10))),
                          material=ground))
    light = quad((-0.75, 4.0, -0.75), (0.75, 4.0, -0.75), (0.75, 4.0, 0.75), (-0.75, 4.0, 0.75))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(light), material=lightmat, emissive=True, le=(20.0, 20.0, 20.0)))
    settings = RenderSettings(N.INTEGRATOR_VOL_PATH, N.METHOD_MIS, N.STRATEGY_UNIFORM, max_depth=32, min_depth=3,
                              rr_threshold=0.99, spp=512, seed=1)
    return s, settings


def displaced_box(n: int, seed: int, amplitude: float = 0.05, frequency: float = 2.5) -> Mesh:
    """Unit cube with n x n quads per face (12 n^2 triangles), each vertex pushed out
    along its ray from the centre by 1 + amplitude * noise."""
    sph = displaced_sphere(n, seed, amplitude=0.0)
    d = sph.positions.astype(np.float64)
    cube = d / np.abs(d).max(1, keepdims=True)
    r = 1.0 + amplitude * value_noise(cube * frequency, seed + 1)
    return Mesh((cube * r[:, None]).astype(np.float32), sph.indices)


def batch_scene(i: int, seed: int = 11):
    """Scene i of the batched workload: one displaced sphere or box with a
    log-uniform triangle count in [10k, 2M] and a diffuse / GGX conductor /
    rough dielectric material on a diffuse ground, lit by a quad light or a
    Gaussian-lobe environment; resolution in {128 ... 1024}, spp in [16, 256],
    max depth in [4, 16]."""
    rng = np.random.default_rng(seed * 1000 + i)
    tris = math.exp(rng.uniform(math.log(1e4), math.log(2e6)))
    n = max(2, int(round(math.sqrt(tris / 12.0))))
    res = [128, 256, 384, 512, 768, 1024]
    w = int(rng.choice(res))
    h = int(rng.choice([r for r in res if r <= w] or [w]))
    spp = int(round(math.exp(rng.uniform(math.log(16), math.log(256)))))
    depth = int(rng.integers(4, 17))
    s = SceneDesc(camera=Camera.look_at(w, h, 40.0, (0.0, 1.8, 4.2), (0.0, 0.9, 0.0)), name=f"batch{i}")
    zero = s.add_const(0.0)
    one = s.add_const(1.0)
    kind = int(rng.integers(0, 3))
    if kind == 0:
        albedo = tuple(float(x) for x in rng.uniform(0.2, 0.8, 3))
        mat = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const(albedo)))
    elif kind == 1:
        rough = s.add_const(math.sqrt(float(rng.uniform(0.05, 0.5))))
        mat = s.add_material(Material(N.MAT_ROUGH_METAL, N.DIST_GGX, tex_roughness=rough, tex_anisotropic=zero,
                                      eta=CU_ETA, k=CU_K))
    else:
        rough = s.add_const(math.sqrt(float(rng.uniform(0.05, 0.5))))
        mat = s.add_material(Material(N.MAT_ROUGH_GLASS, N.DIST_GGX, tex_r=one, tex_t=one, tex_roughness=rough,
                                      tex_anisotropic=zero, eta_a=1.0, eta_b=1.5))
    shape = displaced_sphere(n, seed + i) if rng.uniform() < 0.5 else displaced_box(n, seed + i)
    shape = shape.transformed(Mat4.scale((0.8, 0.8, 0.8)) * Mat4.translation((0.0, 0.9, 0.0)))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(shape), material=mat))
    ground = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const((0.5, 0.5, 0.5))))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(quad((-10, 0, -10), (-10, 0, 10), (10, 0, 10), (10, 0, -10))),
                          material=ground))
    if rng.uniform() < 0.5:
        lm = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const((0.5, 0.5, 0.5))))
        light = quad((-0.6, 3.5, -0.6), (0.6, 3.5, -0.6), (0.6, 3.5, 0.6), (-0.6, 3.5, 0.6))
        s.groups.append(Group(N.GROUP_MESH, s.add_mesh(light), material=lm, emissive=True, le=(25.0, 25.0, 25.0)))
    else:
        env = s.add_texture(gaussian_lobe_env(128, 64, seed + i))
        s.groups.append(Group(N.GROUP_INFINITE_LIGHT, env))
    settings = RenderSettings(N.INTEGRATOR_PATH, N.METHOD_MIS, N.STRATEGY_UNIFORM, max_depth=depth, min_depth=3,
                              rr_threshold=0.99, spp=spp, seed=1 + i)
    return s, settings


def batch_scenes(count: int = 32, seed: int = 11):
    """The batched workload: `count` independent scenes (batch_scene)."""
    return [batch_scene(i, seed) for i in range(count)]


def albedo_image(size: int, seed: int, lo: float = 0.15, hi: float = 0.85) -> np.ndarray:
    """size x size x 3 smooth colour field in [lo, hi] (value noise per channel), img[y, x, c]."""
    ys, xs = np.meshgrid(np.arange(size) / size, np.arange(size) / size, indexing="ij")
    pts = np.stack([xs.reshape(-1) * 6.0, ys.reshape(-1) * 6.0, np.zeros(size * size)], 1)
    img = np.empty((size * size, 3))
    for c in range(3):
        n = value_noise(pts + 17.0 * c, seed + c)
        img[:, c] = lo + (hi - lo) * (0.5 + 0.5 * np.clip(n, -1.0, 1.0))
    return img.reshape(size, size, 3).astype(np.float32)


def adjoint_patches(width=256, height=256, sphere_n=129, tex_size=512, patches=(8, 8), seed=5, alpha=None,
                    albedo_seed=None):
    """The adjoint workload: the displaced sphere of the instanced workload (one
    instance, 12 * 129^2 triangles) with spherical UVs, cut into 8 x 8 patches by
    (theta, phi) of the triangle centroids; each patch is a GGX rough_plastic with
    its own alpha and the shared albedo texture (tex_size^2 RGB, Clamp/Nearest);
    Gaussian-lobe environment.  Returns (scene, settings, params) where params
    holds the albedo texture index and the alpha material indices / values."""
    rng = np.random.default_rng(seed)
    s = SceneDesc(camera=Camera.look_at(width, height, 35.0, (0.0, 0.9, 3.6), (0.0, 0.0, 0.0)), name="adjoint")
    sph = displaced_sphere(sphere_n, 7)
    p = sph.positions.astype(np.float64)
    d = p / np.linalg.norm(p, axis=1, keepdims=True)
    uv = np.stack([np.arctan2(d[:, 0], -d[:, 2]) / (2 * math.pi) + 0.5,
                   np.arccos(np.clip(d[:, 1], -1, 1)) / math.pi], 1).astype(np.float32)
    cen = d[sph.indices].mean(1)
    cen /= np.linalg.norm(cen, axis=1, keepdims=True)
    th = np.arccos(np.clip(cen[:, 1], -1, 1)) / math.pi
    ph = np.arctan2(cen[:, 0], -cen[:, 2]) / (2 * math.pi) + 0.5
    nt, nph = patches
    patch = np.minimum((th * nt).astype(int), nt - 1) * nph + np.minimum((ph * nph).astype(int), nph - 1)
    if albedo_seed is None:
        albedo_seed = seed + 100
    tex = s.add_texture(Texture.from_image_hw3(albedo_image(tex_size, albedo_seed)))
    zero = s.add_const(0.0)
    if alpha is None:
        alpha = rng.uniform(0.05, 0.5, nt * nph)
    mats = []
    for k in range(nt * nph):
        rough = s.add_const(math.sqrt(float(alpha[k])))
        m = s.add_material(Material(N.MAT_ROUGH_PLASTIC, N.DIST_GGX, tex_r=tex, tex_roughness=rough,
                                    tex_anisotropic=zero))
        mats.append(m)
        sel = np.nonzero(patch == k)[0]
        if sel.size == 0:
            continue
        tri = sph.indices[sel]
        used, inv = np.unique(tri.reshape(-1), return_inverse=True)
        mesh = Mesh(sph.positions[used], inv.reshape(-1, 3).astype(np.int32), None, uv[used])
        s.groups.append(Group(N.GROUP_MESH, s.add_mesh(mesh), material=m))
    env = s.add_texture(gaussian_lobe_env(256, 128, seed))
    s.groups.append(Group(N.GROUP_INFINITE_LIGHT, env))
    settings = RenderSettings(N.INTEGRATOR_PATH, N.METHOD_MIS, N.STRATEGY_UNIFORM, max_depth=6, min_depth=3,
                              rr_threshold=0.99, spp=64, seed=1)
    params = {"albedo_texture": tex, "alpha_materials": mats, "alpha": np.asarray(alpha, dtype=np.float64),
              "roughness_textures": [s.materials[m].tex_roughness for m in mats]}
    return s, settings, params


WORKLOADS = {
    "cornell": cornell_box,
    "instanced": instanced_spheres,
    "volume": volume_sphere,
}


def material_zoo(width=64, height=64, seed=3):
    """Small test scene exercising every material plugin, both area-light shapes,
    instancing and an environment light (parity tests, not a benchmark)."""
    s = SceneDesc(camera=Camera.look_at(width, height, 50.0, (0.0, 1.4, 4.2), (0.0, 0.6, 0.0)), name="zoo")
    zero = s.add_const(0.0)
    one = s.add_const(1.0)
    white = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const((0.7, 0.7, 0.7))))
    checker = np.zeros((8, 8, 3), dtype=np.float32)
    checker[(np.add.outer(np.arange(8), np.arange(8)) % 2) == 0] = (0.8, 0.3, 0.2)
    checker[(np.add.outer(np.arange(8), np.arange(8)) % 2) == 1] = (0.2, 0.3, 0.8)
    ck = s.add_texture(Texture.from_image_hw3(checker, N.WRAP_REPEAT, N.FILTER_LINEAR))
    two = s.add_material(Material(N.MAT_DIFFUSE, tex_r=ck, two_sided=True))
    metal = s.add_material(Material(N.MAT_ROUGH_METAL, N.DIST_GGX, tex_roughness=s.add_const(0.4),
                                    tex_anisotropic=s.add_const(0.3), eta=CU_ETA, k=CU_K))
    metal_b = s.add_material(Material(N.MAT_ROUGH_METAL, N.DIST_BECKMANN, tex_roughness=s.add_const(0.3),
                                      tex_anisotropic=zero, eta=CU_ETA, k=CU_K))
    glass = s.add_material(Material(N.MAT_ROUGH_GLASS, N.DIST_GGX, tex_r=one, tex_t=one, tex_roughness=s.add_const(0.25),
                                    tex_anisotropic=zero, eta_a=1.0, eta_b=1.5))
    plastic = s.add_material(Material(N.MAT_ROUGH_PLASTIC, N.DIST_GGX, tex_r=s.add_const((0.2, 0.6, 0.3)),
                                      tex_roughness=s.add_const(0.3), tex_anisotropic=zero, kd=0.6, ks=0.4))
    plastic_b = s.add_material(Material(N.MAT_ROUGH_PLASTIC, N.DIST_BECKMANN, tex_r=s.add_const((0.6, 0.5, 0.2)),
                                        tex_roughness=s.add_const(0.2), tex_anisotropic=s.add_const(-0.4)))
    mirror = s.add_material(Material(N.MAT_PERFECT_MIRROR, tex_r=s.add_const((0.9, 0.9, 0.9))))
    pglass = s.add_material(Material(N.MAT_PERFECT_GLASS, tex_r=one, tex_t=one))
    lightmat = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const(0.5)))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(quad((-3, 0, -3), (-3, 0, 3), (3, 0, 3), (3, 0, -3))), material=two))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(quad((-3, 0, -2), (3, 0, -2), (3, 3, -2), (-3, 3, -2))), material=white))
    from .scene import Sphere
    for i, (m, x) in enumerate([(metal, -1.6), (glass, -0.55), (plastic, 0.55), (pglass, 1.6)]):
        s.spheres.append(Sphere((x, 0.45, 0.0), 0.45))
        s.groups.append(Group(N.GROUP_SPHERE, len(s.spheres) - 1, material=m))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(box_mesh((-1.0, 0.3, 1.1), (0.5, 0.6, 0.5), 25.0)), material=mirror))
    proto = s.add_mesh(displaced_sphere(6, seed, amplitude=0.1))
    s.blas.append([Group(N.GROUP_MESH, proto)])
    for j, (m, x) in enumerate([(metal_b, 0.4), (plastic_b, 1.3)]):
        m2w = Mat4.scale((0.35, 0.35, 0.35)) * Mat4.from_axis_angle((0, 1, 0), 0.7 * j) * Mat4.translation((x, 0.35, 1.2))
        s.groups.append(Group(N.GROUP_INSTANCE, 0, material=m, model_to_world=m2w))
    light = quad((-0.5, 2.8, -0.5), (0.5, 2.8, -0.5), (0.5, 2.8, 0.5), (-0.5, 2.8, 0.5))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(light), material=lightmat, emissive=True, le=(8.0, 8.0, 8.0)))
    s.spheres.append(Sphere((2.2, 2.2, 0.5), 0.15))
    s.groups.append(Group(N.GROUP_SPHERE, len(s.spheres) - 1, material=lightmat, emissive=True, le=(30.0, 20.0, 10.0)))
    env = s.add_texture(gaussian_lobe_env(64, 32, seed, lobes=4))
    s.groups.append(Group(N.GROUP_INFINITE_LIGHT, env, model_to_world=Mat4.from_axis_angle((0, 1, 0), 0.3)))
    settings = RenderSettings(N.INTEGRATOR_PATH, N.METHOD_MIS, N.STRATEGY_UNIFORM, max_depth=6, min_depth=2,
                              rr_threshold=0.99, spp=4, seed=5)
    return s, settings


def volume_box(width=64, height=64, seed=9):
    """Small vol_path test scene: a global medium, a medium-filled displaced sphere
    with no material, a glass sphere, diffuse ground and one area light."""
    s, st = volume_sphere(width, height, sphere_n=6, seed=seed)
    s.global_medium = s.add_medium(Medium((0.01, 0.02, 0.03), (0.05, 0.05, 0.05), g=-0.3, scale=1.0))
    one = s.add_const(1.0)
    zero = s.add_const(0.0)
    glass = s.add_material(Material(N.MAT_ROUGH_GLASS, N.DIST_GGX, tex_r=one, tex_t=one, tex_roughness=s.add_const(0.2),
                                    tex_anisotropic=zero, eta_a=1.0, eta_b=1.5))
    from .scene import Sphere
    s.spheres.append(Sphere((1.6, 0.5, 0.3), 0.5))
    s.groups.append(Group(N.GROUP_SPHERE, len(s.spheres) - 1, material=glass, medium_outside=s.global_medium))
    for g in s.groups:
        if g.kind == N.GROUP_MESH and g.material >= 0:
            g.medium_outside = s.global_medium
    return s, st.replace(spp=4, max_depth=12)
