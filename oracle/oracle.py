"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is the C++ restatement of Radiantium's path-tracing hot path that
the CUDA library is checked against.  Only tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline leg import this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from radiantium_gb300 import native as N

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compiles liboracle.so with the committed Makefile (make -C oracle)."""
    if force or not os.path.exists(LIB):
        subprocess.run(["make", "-C", HERE, "-s"], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.or_scene_create.restype = vp
        L.or_scene_create.argtypes = [C.POINTER(N.SceneDescC), C.c_char_p, C.c_int]
        L.or_scene_destroy.argtypes = [vp]
        L.or_trace_closest.argtypes = [vp, vp, C.c_int64, vp, C.c_int, C.POINTER(N.Stats)]
        L.or_trace_any.argtypes = [vp, vp, C.c_int64, vp, C.c_int, C.POINTER(N.Stats)]
        L.or_render.argtypes = [vp, C.POINTER(N.RenderParams), vp, C.c_int, C.POINTER(N.Stats)]
        L.or_render_samples.argtypes = [vp, C.POINTER(N.RenderParams), vp, C.c_int]
        L.or_render_particles.argtypes = [vp, C.POINTER(N.RenderParams), C.c_int64, C.c_int64, vp, C.c_int,
                                          C.POINTER(N.Stats)]
        L.or_particle_splats.argtypes = [vp, C.POINTER(N.RenderParams), C.c_int64, C.c_int64, C.c_int, vp, vp, vp,
                                         C.c_int]
        L.or_camera_rays.argtypes = [vp, vp, C.c_int64, vp]
        L.or_bvh.argtypes = [vp, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64), vp, vp, vp, vp, vp]
        L.or_scene_lights.argtypes = [vp, C.POINTER(C.c_int64), vp, vp, vp]
        L.or_detmath.argtypes = [C.c_int, vp, vp, vp, C.c_int64]
        L.or_philox.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, vp]
        L.or_philox_raw.argtypes = [vp, vp, vp]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class OracleScene:
    """The restated Scene built from a SceneDesc."""

    def __init__(self, scene):
        self.packed = scene.to_c()
        err = C.create_string_buffer(512)
        self.h = lib().or_scene_create(C.byref(self.packed.desc), err, 512)
        if not self.h:
            raise ValueError("oracle scene: " + err.value.decode())
        self.scene = scene

    def close(self):
        if self.h:
            lib().or_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace_closest(self, rays: np.ndarray, threads: int = 0, stats: bool = False):
        """Scene.Intersect per ray; with stats, also the summed traversal counters."""
        rays = np.ascontiguousarray(rays, dtype=N.ray_dtype())
        hits = np.zeros(rays.shape[0], dtype=N.hit_dtype())
        st = N.Stats()
        rc = lib().or_trace_closest(self.h, _ptr(rays), rays.shape[0], _ptr(hits), threads,
                                    C.byref(st) if stats else None)
        if rc != 0:
            raise N.RTError(rc, "oracle trace_closest")
        return (hits, st.as_dict()) if stats else hits

    def trace_any(self, rays: np.ndarray, threads: int = 0, stats: bool = False):
        """Scene.IsOccluded-style any hit per ray; with stats, also the summed traversal counters."""
        rays = np.ascontiguousarray(rays, dtype=N.ray_dtype())
        occ = np.zeros(rays.shape[0], dtype=np.uint8)
        st = N.Stats()
        rc = lib().or_trace_any(self.h, _ptr(rays), rays.shape[0], _ptr(occ), threads,
                                C.byref(st) if stats else None)
        if rc != 0:
            raise N.RTError(rc, "oracle trace_any")
        return (occ, st.as_dict()) if stats else occ

    def render(self, settings, threads: int = 0, stats: bool = False):
        w = settings.width or (self.scene.camera.width - settings.x0)
        h = settings.height or (self.scene.camera.height - settings.y0)
        out = np.zeros(w * h * 3, dtype=np.float32)
        st = N.Stats()
        p = settings.to_c()
        rc = lib().or_render(self.h, C.byref(p), _ptr(out), threads, C.byref(st) if stats else None)
        if rc != 0:
            raise N.RTError(rc, "oracle render")
        img = out.reshape(w, h, 3)
        return (img, st.as_dict()) if stats else img

    def render_samples(self, settings, threads: int = 0) -> np.ndarray:
        w = settings.width or (self.scene.camera.width - settings.x0)
        h = settings.height or (self.scene.camera.height - settings.y0)
        out = np.zeros(w * h * settings.spp * 3, dtype=np.float32)
        p = settings.to_c()
        rc = lib().or_render_samples(self.h, C.byref(p), _ptr(out), threads)
        if rc != 0:
            raise N.RTError(rc, "oracle render_samples")
        return out.reshape(w, h, settings.spp, 3)

    def render_particles(self, settings, count: int, first: int = 0, threads: int = 0, stats: bool = False):
        """AdjointParticleRenderer film of particles [first, first + count): (width, height, 3)."""
        cam = self.scene.camera
        out = np.zeros(cam.width * cam.height * 3, dtype=np.float32)
        st = N.Stats()
        p = settings.to_c()
        rc = lib().or_render_particles(self.h, C.byref(p), first, count, _ptr(out), threads,
                                       C.byref(st) if stats else None)
        if rc != 0:
            raise N.RTError(rc, "oracle render_particles")
        img = out.reshape(cam.width, cam.height, 3)
        return (img, st.as_dict()) if stats else img

    def particle_splats(self, settings, count: int, max_per: int, first: int = 0, threads: int = 0):
        """Camera connections per particle: (n[count], pix[count, max_per], rgb[count, max_per, 3])."""
        n = np.zeros(count, dtype=np.int32)
        pix = np.zeros((count, max_per), dtype=np.int32)
        rgb = np.zeros((count, max_per, 3), dtype=np.float32)
        p = settings.to_c()
        rc = lib().or_particle_splats(self.h, C.byref(p), first, count, max_per, _ptr(n), _ptr(pix), _ptr(rgb),
                                      threads)
        if rc != 0:
            raise N.RTError(rc, "oracle particle_splats")
        return n, pix, rgb

    def camera_rays(self, screen_pos: np.ndarray) -> np.ndarray:
        sp = np.ascontiguousarray(screen_pos, dtype=np.float32).reshape(-1, 2)
        out = np.zeros(sp.shape[0], dtype=N.ray_dtype())
        lib().or_camera_rays(self.h, _ptr(sp), sp.shape[0], _ptr(out))
        return out

    def bvh(self, which: int = -1) -> dict:
        nn, npr = C.c_int64(), C.c_int64()
        lib().or_bvh(self.h, which, C.byref(nn), C.byref(npr), None, None, None, None, None)
        b = np.zeros((nn.value, 6), dtype=np.float32)
        idx = np.zeros(nn.value, dtype=np.int32)
        cnt = np.zeros(nn.value, dtype=np.int32)
        ax = np.zeros(nn.value, dtype=np.int32)
        order = np.zeros(npr.value, dtype=np.int32)
        lib().or_bvh(self.h, which, C.byref(nn), C.byref(npr), _ptr(b), _ptr(idx), _ptr(cnt), _ptr(ax), _ptr(order))
        return {"bounds": b, "index": idx, "count": cnt, "axis": ax, "prim_order": order}

    def lights(self) -> dict:
        """Scene.Lights in order: kind (0 area, 1 infinite), carrying primitive id, radiance."""
        n = C.c_int64()
        lib().or_scene_lights(self.h, C.byref(n), None, None, None)
        kind = np.zeros(n.value, dtype=np.int32)
        prim = np.zeros(n.value, dtype=np.int32)
        le = np.zeros((n.value, 3), dtype=np.float32)
        lib().or_scene_lights(self.h, C.byref(n), _ptr(kind), _ptr(prim), _ptr(le))
        return {"kind": kind, "prim": prim, "le": le}


DETMATH_FN = {"sin": 0, "cos": 1, "tan": 2, "atan": 3, "atan2": 4, "acos": 5, "exp": 6, "log": 7}


def detmath(fn: str, a: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b if b is not None else a, dtype=np.float32)
    out = np.empty_like(a)
    rc = lib().or_detmath(DETMATH_FN[fn], _ptr(a), _ptr(b), _ptr(out), a.size)
    if rc != 0:
        raise ValueError(fn)
    return out


def philox_stream(seed: int, x: int, y: int, s: int, count: int) -> np.ndarray:
    out = np.zeros(count, dtype=np.uint32)
    lib().or_philox(seed, x, y, s, count, _ptr(out))
    return out


def philox_raw(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().or_philox_raw(_ptr(c), _ptr(k), _ptr(out))
    return out
