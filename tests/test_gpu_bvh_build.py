"""The GPU builder (rt_bvh_gpu.cu) against the host builder (gpu).

Both must produce the reference's SAH tree: every node (bounds bits, child /
first-slot index, primitive count, split axis) and the primitive order of
the leaves, for random boxes, duplicate-heavy and degenerate inputs and the
triangle boxes of a mesh, and a scene uploaded with trees built on the GPU
must render the same film as with trees built on the host.
"""
import ctypes as C

import numpy as np
import pytest

from radiantium_gb300 import native as N
from radiantium_gb300 import procedural
from radiantium_gb300.device import Device
from tests.test_cpu_oracle import _lib_bvh, _tri_boxes

pytestmark = pytest.mark.gpu


def _gpu_bvh(dev, boxes, max_prims=1):
    f = dev.lib.rt_debug_bvh_gpu
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_int64)] + [C.c_void_p] * 6
    boxes = np.ascontiguousarray(boxes, dtype=np.float32)
    n = boxes.shape[0]
    nn = C.c_int64()
    assert f(dev.h, boxes.ctypes.data, n, max_prims, C.byref(nn), None, None, None, None, None, None) == 0
    b = np.zeros((nn.value, 6), np.float32)
    idx, cnt, ax = (np.zeros(nn.value, np.int32) for _ in range(3))
    order = np.zeros(n, np.int32)
    depth = C.c_int32()
    assert f(dev.h, boxes.ctypes.data, n, max_prims, C.byref(nn), b.ctypes.data, idx.ctypes.data, cnt.ctypes.data,
             ax.ctypes.data, order.ctypes.data, C.byref(depth)) == 0
    return {"bounds": b, "index": idx, "count": cnt, "axis": ax, "prim_order": order}


def _same(g, h):
    assert g["bounds"].shape == h["bounds"].shape
    for k in ("index", "count", "axis", "prim_order"):
        assert np.array_equal(g[k], h[k]), k
    assert np.array_equal(g["bounds"].view(np.uint32), h["bounds"].view(np.uint32))


def _random_boxes(n, seed, dup=False):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-10, 10, (n, 3))
    if dup:
        c = np.round(c / 4) * 4                 # many identical centroids
    e = rng.uniform(0.001, 0.5, (n, 3))
    return np.concatenate([c - e, c + e], 1).astype(np.float32)


@pytest.mark.parametrize("n", [1, 2, 3, 17, 1000, 40000])
@pytest.mark.parametrize("max_prims", [1, 4])
def test_random_boxes(dev, n, max_prims):
    b = _random_boxes(n, n + max_prims)
    _same(_gpu_bvh(dev, b, max_prims), _lib_bvh(b, max_prims))


@pytest.mark.parametrize("max_prims", [1, 3])
def test_duplicates_and_degenerate(dev, max_prims):
    b = _random_boxes(5000, 7, dup=True)
    _same(_gpu_bvh(dev, b, max_prims), _lib_bvh(b, max_prims))
    flat = np.tile(np.array([[0, 0, 0, 1, 1, 1]], np.float32), (64, 1))        # one centroid: a single leaf
    _same(_gpu_bvh(dev, flat, max_prims), _lib_bvh(flat, max_prims))
    line = np.zeros((300, 6), np.float32)                                     # centroids on one axis
    line[:, 0] = np.arange(300) * 0.5
    line[:, 3] = line[:, 0] + 0.25
    line[:, 4] = line[:, 5] = 0.1
    _same(_gpu_bvh(dev, line, max_prims), _lib_bvh(line, max_prims))


def test_mesh_boxes(dev):
    b = _tri_boxes(procedural.displaced_sphere(60, 3))
    _same(_gpu_bvh(dev, b, 1), _lib_bvh(b, 1))


def test_scene_built_on_the_gpu_renders_the_same():
    s, st = procedural.instanced_spheres(96, 96, sphere_n=40, grid=3, env_w=32, env_h=16)
    films = []
    for min_prims in (0, 1):                     # 0: host builder only; 1: every tree on the GPU
        d = Device(0)
        try:
            f = d.lib.rt_debug_set_gpu_build
            f.argtypes = [C.c_void_p, C.c_int]
            assert f(d.h, min_prims) == 0
            d.upload(s)
            films.append(d.render(st.replace(spp=4)))
        finally:
            d.close()
    assert np.array_equal(films[0].view(np.uint32), films[1].view(np.uint32))
