"""Python binding of the CUDA library through its C ABI (include/radiantium.h).

:class:`Device` owns one rt context (one CUDA stream) and one uploaded scene.
Every call goes through ``libradiantium_gb300.so``; a missing library raises
(there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import native as N
from .scene import RenderSettings, SceneDesc


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class Device:
    """An rt context on one GPU: upload a scene, trace ray batches, render."""

    def __init__(self, device: int = 0):
        self.lib = N.load_library()
        h = C.c_void_p()
        rc = self.lib.rt_create(device, C.byref(h))
        if rc != N.RT_OK:
            raise N.RTError(rc, "rt_create failed (is a CUDA device visible?)")
        self.h = h
        self.scene: SceneDesc | None = None
        self._packed = None

    def _check(self, rc: int):
        if rc != N.RT_OK:
            raise N.RTError(rc, self.lib.rt_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.lib.rt_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload(self, scene: SceneDesc):
        packed = scene.to_c()
        self._check(self.lib.rt_upload_scene(self.h, C.byref(packed.desc)))
        self.scene, self._packed = scene, packed

    def set_counting(self, on: bool):
        self._check(self.lib.rt_set_counting(self.h, 1 if on else 0))

    def set_renderer(self, mode: int):
        """N.RENDERER_AUTO / RENDERER_MEGAKERNEL / RENDERER_WAVEFRONT"""
        self._check(self.lib.rt_set_renderer(self.h, mode))

    def set_traversal(self, mode: int):
        """N.TRAVERSAL_EXACT (the reference's tree and order) / N.TRAVERSAL_WIDE (opt-in fast traversal)"""
        self._check(self.lib.rt_set_traversal(self.h, mode))

    def traversal(self) -> int:
        """The traversal the next call will run (WIDE only where the uploaded scene allows it)."""
        v = C.c_int()
        self._check(self.lib.rt_get_traversal(self.h, C.byref(v)))
        return v.value

    def set_light_sampling(self, mode: int):
        """N.LIGHT_SAMPLING_CDF (the reference's CDF search) / N.LIGHT_SAMPLING_ALIAS (opt-in alias tables
        with the same texel pmf) for the infinite lights of this context's scene"""
        self._check(self.lib.rt_set_light_sampling(self.h, mode))

    def light_sampling(self) -> int:
        v = C.c_int()
        self._check(self.lib.rt_get_light_sampling(self.h, C.byref(v)))
        return v.value

    def env_sample(self, u, which=0):
        """Texel offsets (column, row) and pdf that infinite light `which` samples for each row
        (u_column, u_row) of u, computed on the device in the current light-sampling mode."""
        u = np.ascontiguousarray(u, np.float32).reshape(-1, 2)
        texel = np.empty((u.shape[0], 2), np.int32)
        pdf = np.empty(u.shape[0], np.float32)
        self._check(self.lib.rt_debug_env_sample(self.h, which, u.ctypes.data, u.shape[0], texel.ctypes.data,
                                                 pdf.ctypes.data))
        return texel, pdf

    def stats(self) -> dict:
        st = N.Stats()
        self._check(self.lib.rt_get_stats(self.h, C.byref(st)))
        return st.as_dict()

    def cancel(self):
        self._check(self.lib.rt_cancel(self.h))

    def trace_closest(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=N.ray_dtype())
        hits = np.zeros(rays.shape[0], dtype=N.hit_dtype())
        self._check(self.lib.rt_trace_closest(self.h, _ptr(rays), rays.shape[0], _ptr(hits)))
        return hits

    def trace_any(self, rays: np.ndarray) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=N.ray_dtype())
        occ = np.zeros(rays.shape[0], dtype=np.uint8)
        self._check(self.lib.rt_trace_any(self.h, _ptr(rays), rays.shape[0], _ptr(occ)))
        return occ

    def _crop(self, s: RenderSettings):
        cam = self.scene.camera
        return (s.width or cam.width - s.x0), (s.height or cam.height - s.y0)

    def render(self, settings: RenderSettings) -> np.ndarray:
        """Averaged film of the crop, ColorBuffer layout (x, y, rgb)."""
        w, h = self._crop(settings)
        out = np.zeros(w * h * 3, dtype=np.float32)
        p = settings.to_c()
        self._check(self.lib.rt_render(self.h, C.byref(p), _ptr(out)))
        return out.reshape(w, h, 3)

    def render_device(self, settings: RenderSettings, out_ptr: int, stream: int = 0):
        """Film written to device memory `out_ptr` (w*h*3 float32) on `stream` (0 = context stream)."""
        p = settings.to_c()
        self._check(self.lib.rt_render_device(self.h, C.byref(p), C.c_void_p(out_ptr), C.c_void_p(stream or None)))

    def render_particles(self, settings: RenderSettings, count: int, first: int = 0) -> np.ndarray:
        """Light-traced film ("adjoint_particle") of particles [first, first + count),
        the whole film in ColorBuffer layout (x, y, rgb)."""
        cam = self.scene.camera
        out = np.zeros(cam.width * cam.height * 3, dtype=np.float32)
        p = settings.to_c()
        self._check(self.lib.rt_render_particles(self.h, C.byref(p), first, count, _ptr(out)))
        return out.reshape(cam.width, cam.height, 3)

    def render_particles_device(self, settings: RenderSettings, count: int, out_ptr: int, first: int = 0,
                                stream: int = 0):
        """Same, film written to device memory `out_ptr` (ScreenX*ScreenY*3 float32)."""
        p = settings.to_c()
        self._check(self.lib.rt_render_particles_device(self.h, C.byref(p), first, count, C.c_void_p(out_ptr),
                                                        C.c_void_p(stream or None)))

    def particle_splats(self, settings: RenderSettings, count: int, max_per: int, first: int = 0):
        """Parity hook: each particle's camera connections, (n[count], pix[count, max_per],
        rgb[count, max_per, 3]) with pix = x * ScreenY + y (-1 past n)."""
        n = np.zeros(count, dtype=np.int32)
        pix = np.zeros((count, max_per), dtype=np.int32)
        rgb = np.zeros((count, max_per, 3), dtype=np.float32)
        p = settings.to_c()
        self._check(self.lib.rt_debug_particle_splats(self.h, C.byref(p), first, count, max_per, _ptr(n), _ptr(pix),
                                                      _ptr(rgb)))
        return n, pix, rgb

    def adjoint_forward(self, settings: RenderSettings) -> np.ndarray:
        """The film the gradients refer to (same as render)."""
        w, h = self._crop(settings)
        out = np.zeros(w * h * 3, dtype=np.float32)
        p = settings.to_c()
        self._check(self.lib.rt_adjoint_forward(self.h, C.byref(p), _ptr(out)))
        return out.reshape(w, h, 3)

    def adjoint_backward(self, settings: RenderSettings, dl_dimage: np.ndarray, albedo_texture: int = -1,
                         alpha_materials=()):
        """Gradient of sum(dl_dimage * I) w.r.t. the albedo texture's texels ((w, h, 3),
        ColorBuffer layout) and the alpha of each listed material."""
        w, h = self._crop(settings)
        dl = np.ascontiguousarray(dl_dimage, dtype=np.float32).reshape(-1)
        if dl.size != w * h * 3:
            raise ValueError("dl_dimage must have the crop's w * h * 3 values")
        mats = np.ascontiguousarray(alpha_materials, dtype=np.int32)
        desc = N.AdjointDesc(albedo_texture, len(mats), mats.ctypes.data_as(C.POINTER(C.c_int32)))
        if albedo_texture >= 0:
            t = self.scene.textures[albedo_texture]
            g_alb = np.zeros(t.width * t.height * 3, dtype=np.float32)
        else:
            t, g_alb = None, np.zeros(3, dtype=np.float32)
        g_alpha = np.zeros(max(1, len(mats)), dtype=np.float32)
        p = settings.to_c()
        self._check(self.lib.rt_adjoint_backward(self.h, C.byref(p), C.byref(desc), _ptr(dl), _ptr(g_alb),
                                                 _ptr(g_alpha)))
        return (g_alb.reshape(t.width, t.height, 3) if t is not None else None), g_alpha[:len(mats)]

    def update_texture(self, index: int, data: np.ndarray):
        """New texels (ColorBuffer layout) for texture `index` of the uploaded scene."""
        t = self.scene.textures[index]
        d = np.ascontiguousarray(data, dtype=np.float32).reshape(-1)
        if d.size != t.width * t.height * 3:
            raise ValueError("texel count mismatch")
        self._check(self.lib.rt_update_texture(self.h, index, _ptr(d)))
        t.data = d.copy()

    def autotune(self, items) -> dict:
        """Picks the fastest film-preserving wavefront settings for this batch
        (rt_autotune); they stay on this context."""
        outs, arr = [], (N.BatchItem * len(items))()
        for i, (d, st) in enumerate(items):
            w, h = d._crop(st)
            out = np.zeros(w * h * 3, dtype=np.float32)
            outs.append(out)
            arr[i].scene_ctx = d.h
            arr[i].params = st.to_c()
            arr[i].out_rgb = out.ctypes.data
        r = N.TuneResult()
        self._check(self.lib.rt_autotune(self.h, arr, len(items), C.byref(r)))
        return {"capacity": r.capacity, "refill": r.refill, "renderer": r.renderer, "ms": r.ms,
                "ms_default": r.ms_default}

    def render_batch(self, items) -> list:
        """Renders [(Device holding the scene, RenderSettings), ...] as one wavefront
        on this device's context; returns the averaged films (x, y, rgb)."""
        outs, arr = [], (N.BatchItem * len(items))()
        for i, (d, st) in enumerate(items):
            w, h = d._crop(st)
            out = np.zeros(w * h * 3, dtype=np.float32)
            outs.append(out.reshape(w, h, 3))
            arr[i].scene_ctx = d.h
            arr[i].params = st.to_c()
            arr[i].out_rgb = out.ctypes.data
        self._check(self.lib.rt_render_batch(self.h, arr, len(items)))
        return outs

    def render_batch_device(self, items, out_ptrs, stream: int = 0):
        """Same as render_batch with each film written to device memory out_ptrs[i] on `stream`."""
        arr = (N.BatchItem * len(items))()
        for i, ((d, st), ptr) in enumerate(zip(items, out_ptrs)):
            arr[i].scene_ctx = d.h
            arr[i].params = st.to_c()
            arr[i].out_rgb = ptr
        self._check(self.lib.rt_render_batch_device(self.h, arr, len(items), C.c_void_p(stream or None)))

    def render_device_noalloc(self, settings: RenderSettings, out_ptr: int, stream: int = 0):
        """Same film as render_device, rendered out of the library's fixed device
        scratch (RT_NOALLOC_SCRATCH_BYTES) with no device allocation."""
        p = settings.to_c()
        self._check(self.lib.rt_render_device_noalloc(self.h, C.byref(p), C.c_void_p(out_ptr),
                                                      C.c_void_p(stream or None)))

    def trace_closest_device(self, rays_ptr: int, n: int, hits_ptr: int, stream: int = 0):
        self._check(self.lib.rt_trace_closest_device(self.h, C.c_void_p(rays_ptr), n, C.c_void_p(hits_ptr),
                                                     C.c_void_p(stream or None)))

    def detmath(self, fn: int, a: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
        """Runs the deterministic math (fn 0..7) or CUDA's own functions (fn 100..107) on the GPU."""
        f = self.lib.rt_debug_detmath
        f.restype = C.c_int
        f.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64]
        a = np.ascontiguousarray(a, dtype=np.float32)
        b = np.ascontiguousarray(a if b is None else b, dtype=np.float32)
        out = np.empty_like(a)
        self._check(f(self.h, fn, _ptr(a), _ptr(b), _ptr(out), a.size))
        return out
