"""The reference's own example scenes on the GPU (gpu).

Every scene of tests/fixtures/reference (Radiantium's Example/**.json with
their OBJ meshes, copied byte for byte) is loaded through the reference's
JSON schema and rendered through the C ABI:

  * path and vol_path scenes: a 32 x 32 crop at the film's centre, 8 spp, on
    the megakernel and both wavefront loop drivers, equal bit for bit to the
    committed oracle film (tests/golden/reference_scenes.npz) and to the
    oracle run here, with equal ray and traversal counters;
  * light-tracer scenes ("adjoint_particle"): the camera connections of 256
    particles equal the committed oracle splats bit for bit.
"""
import os

import numpy as np
import pytest

from radiantium_gb300 import native as N
from oracle.oracle import OracleScene
from tests.golden import make_golden

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_scenes.npz")
COUNTERS = ("samples", "rays_closest", "rays_shadow", "node_visits", "prim_tests", "instance_visits")
CASES = make_golden.reference_scene_cases()


@pytest.fixture(scope="module")
def golden():
    with np.load(GOLDEN, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


@pytest.mark.parametrize("case", [c for c in CASES if c[2].integrator != N.INTEGRATOR_PARTICLE], ids=lambda c: c[0])
def test_reference_scene_crop_equals_oracle(dev, golden, case):
    name, scene, st = case
    want = golden[name + "_film"]
    dev.upload(scene)
    orc = OracleScene(scene)
    try:
        o, oc = orc.render(st, stats=True)
    finally:
        orc.close()
    assert np.array_equal(o.view(np.uint32), want), "the oracle reproduces its committed film"
    dev.set_counting(True)
    try:
        for mode in (N.RENDERER_MEGAKERNEL, N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH):
            dev.set_renderer(mode)
            g = dev.render(st)
            gc = dev.stats()
            assert np.array_equal(g.view(np.uint32), want), (name, mode, float(np.abs(g - o).max()))
            if mode != N.RENDERER_WAVEFRONT_GRAPH:
                for k in COUNTERS:
                    assert gc[k] == oc[k], (name, mode, k, gc[k], oc[k])
    finally:
        dev.set_counting(False)
        dev.set_renderer(N.RENDERER_AUTO)


@pytest.mark.parametrize("case", [c for c in CASES if c[2].integrator == N.INTEGRATOR_PARTICLE], ids=lambda c: c[0])
def test_reference_scene_particles_equal_oracle(dev, golden, case):
    name, scene, st = case
    dev.upload(scene)
    n, pix, rgb = dev.particle_splats(st, 256, 12, first=77)
    assert np.array_equal(n, golden[name + "_n"])
    assert np.array_equal(pix, golden[name + "_pix"])
    assert np.array_equal(rgb.view(np.uint32), golden[name + "_rgb"])
    assert n.sum() > 0
