"""The benchmark geometries at full size against the oracle (gpu).

The timed workloads trace trees that the GPU builder makes (every tree of
32 Ki primitives or more): the 199,692-triangle prototype of the 64-instance
scene, the 499,392-triangle medium sphere of the vol_path scene and the
1,572,528-triangle mesh of the largest of the 32 batched scenes.  These tests
tie those trees, and what is traced and rendered through them, to the oracle's
restatement of the reference (Accelerators/Bvh.cs:234-442 for the build,
:126-232 for the traversals, Integrators/PathTracer.cs and
VolumetricPathTracer.cs for the films):

  * the device-built tree equals the oracle's tree node for node (bounds
    bits, child / first-slot index, primitive count, split axis) and in leaf
    order;
  * 100 k rays (camera rays and random rays through the scene's box) give the
    oracle's closest hits (primitive id, instance id, t, u, v and tie flags
    bit for bit), any-hit answers, and node / primitive / instance visit
    counts;
  * 32 x 32 crops at the centre and a corner of the full-resolution films
    (1024 x 1024 and 512 x 512) equal the oracle's films bit for bit, with
    equal ray and traversal counters, on the megakernel and the wavefront.
"""
import numpy as np
import pytest

from radiantium_gb300 import native as N
from radiantium_gb300 import procedural
from oracle.oracle import OracleScene
from tests.test_gpu_bvh_build import _gpu_bvh
from tests.test_gpu_parity import assert_hits_equal, random_rays
from tests.test_cpu_oracle import _tri_boxes

pytestmark = pytest.mark.gpu

TRAVERSAL = ("node_visits", "prim_tests", "instance_visits")
RENDER_COUNTERS = ("samples", "rays_closest", "rays_shadow") + TRAVERSAL


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _scene(name):
    if name == "C2":
        return procedural.instanced_spheres()
    if name == "C3":
        return procedural.volume_sphere()
    return procedural.batch_scene(8)          # the largest of the 32 batched scenes


@pytest.fixture(scope="module")
def scenes():
    cache = {}

    def get(name):
        if name not in cache:
            s, st = _scene(name)
            cache[name] = (s, st, OracleScene(s))
        return cache[name]
    yield get
    for _, _, o in cache.values():
        o.close()


def _same_tree(g, o):
    assert g["bounds"].shape == o["bounds"].shape, (g["bounds"].shape, o["bounds"].shape)
    for k in ("index", "count", "axis", "prim_order"):
        assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(_bits(g["bounds"]), _bits(o["bounds"]))


@pytest.mark.parametrize("name", ["C2", "C3", "C4"])
def test_device_tree_equals_oracle_tree(dev, scenes, name):
    s, _, orc = scenes(name)
    if name == "C2":
        boxes, which = _tri_boxes(s.meshes[s.blas[0][0].ref]), 0          # the instanced prototype
    else:
        boxes = np.concatenate([_tri_boxes(s.meshes[g.ref]) for g in s.groups if g.kind == N.GROUP_MESH])
        which = -1
    assert boxes.shape[0] >= 32 * 1024, "the upload builds this tree on the GPU"
    _same_tree(_gpu_bvh(dev, boxes, 1), orc.bvh(which))


def _rays(s, orc, n, seed):
    """Half camera rays through random film positions, half random rays aimed
    into the scene's bounding box from around it and from inside it."""
    rng = np.random.default_rng(seed)
    cam = s.camera
    pos = rng.random((n // 2, 2)) * np.array([cam.width, cam.height])
    cam_rays = orc.camera_rays(pos)
    root = orc.bvh(-1)["bounds"][0].astype(np.float64)
    box = (root[:3], root[3:])
    return np.concatenate([cam_rays, random_rays(box, n // 4, seed + 1),
                           random_rays(box, n - n // 2 - n // 4, seed + 2, inside=True)])


@pytest.mark.parametrize("name", ["C2", "C3", "C4"])
def test_ray_batches_equal_oracle(dev, scenes, name):
    s, _, orc = scenes(name)
    dev.upload(s)
    rays = _rays(s, orc, 100000, 40)
    dev.set_counting(True)
    try:
        g = dev.trace_closest(rays)
        gc = dev.stats()
        ga = dev.trace_any(rays)
        gac = dev.stats()
    finally:
        dev.set_counting(False)
    o, oc = orc.trace_closest(rays, stats=True)
    oa, oac = orc.trace_any(rays, stats=True)
    assert_hits_equal(g, o)
    assert (o["prim"] >= 0).sum() > 20000, "most rays should hit the geometry"
    if name == "C2":
        assert (o["sub"] >= 0).sum() > 10000, "rays should hit instanced prototypes"
    assert np.array_equal(ga, oa)
    for k in TRAVERSAL:
        assert gc[k] == oc[k], ("closest", k, gc[k], oc[k])
        assert gac[k] == oac[k], ("any", k, gac[k], oac[k])


@pytest.mark.parametrize("renderer", [N.RENDERER_MEGAKERNEL, N.RENDERER_WAVEFRONT])
@pytest.mark.parametrize("name", ["C2", "C3"])
def test_full_resolution_crops_equal_oracle(dev, scenes, name, renderer):
    s, st, orc = scenes(name)
    dev.upload(s)
    w, h = s.camera.width, s.camera.height
    spp = 2 if name == "C2" else 1
    for x0, y0 in (((w - 32) // 2, (h - 32) // 2), (0, h - 32)):      # centre and a corner
        crop = st.replace(spp=spp, sample_begin=7, x0=x0, y0=y0, width=32, height=32)
        dev.set_counting(True)
        dev.set_renderer(renderer)
        try:
            g = dev.render(crop)
            gc = dev.stats()
        finally:
            dev.set_counting(False)
            dev.set_renderer(N.RENDERER_AUTO)
        o, oc = orc.render(crop, stats=True)
        assert np.array_equal(_bits(g), _bits(o)), (name, x0, y0, float(np.abs(g - o).max()))
        assert o.mean() > 0
        for k in RENDER_COUNTERS:
            assert gc[k] == oc[k], (name, x0, y0, k, gc[k], oc[k])
