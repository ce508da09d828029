"""Parity at the benchmark configurations' full sizes (gpu).

The oracle cannot render these in test time, so the checks are the
size-independent properties the renderer offers: every renderer computes the
same per-sample values, so a pass over the whole film must be bit-identical
between the plain megakernel, the host-driven wavefront and the graph-driven
wavefront, with identical traversal counters; and a batch must reproduce each
scene's own render.  The light tracer's films agree within the float
summation order of their splats, with identical ray and node counts.

  C2: 64 instances of a 199,692-triangle sphere, 1024 x 1024, 1 spp
  C3: 499,392-triangle medium sphere, 512 x 512, 2 spp (vol_path, depth 32)
  C4: the 32 scenes of the batch at 1 spp each (10 k - 2 M triangles)
  C6: the light tracer's Cornell box at 800 x 600, 4 Mi particles
"""
import numpy as np
import pytest

from radiantium_gb300 import native as N
from radiantium_gb300 import procedural
from radiantium_gb300.device import Device

pytestmark = pytest.mark.gpu
MODES = (N.RENDERER_MEGAKERNEL, N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH)
COUNTERS = ("samples", "rays_closest", "rays_shadow", "node_visits", "prim_tests", "instance_visits")


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _all_renderers(dev, st):
    films, counts = [], []
    dev.set_counting(True)
    try:
        for m in MODES:
            dev.set_renderer(m)
            films.append(dev.render(st))
            counts.append(dev.stats())
    finally:
        dev.set_counting(False)
        dev.set_renderer(N.RENDERER_AUTO)
    return films, counts


@pytest.mark.parametrize("config", ["C2", "C3"])
def test_full_size_pass_identical_across_renderers(dev, config):
    if config == "C2":
        s, st = procedural.instanced_spheres()
        st = st.replace(spp=1, sample_begin=5)
    else:
        s, st = procedural.volume_sphere()
        st = st.replace(spp=2, sample_begin=9)
    dev.upload(s)
    films, counts = _all_renderers(dev, st)
    assert films[0].shape == (s.camera.width, s.camera.height, 3)
    assert np.isfinite(films[0]).all() and films[0].mean() > 0
    for m, f, c in zip(MODES[1:], films[1:], counts[1:]):
        assert np.array_equal(_bits(f), _bits(films[0])), (config, m, float(np.abs(f - films[0]).max()))
        if m == N.RENDERER_WAVEFRONT:
            for k in COUNTERS:
                assert c[k] == counts[0][k], (config, k, c[k], counts[0][k])


def test_full_batch_reproduces_each_scene():
    """C4's 32 scenes in one wavefront at 1 spp each: every film equals the scene's own render."""
    scenes = procedural.batch_scenes()
    devs = []
    try:
        for s, _ in scenes:
            d = Device(0)
            d.upload(s)
            devs.append(d)
        host = Device(0)
        items = [(d, st.replace(spp=1, sample_begin=3)) for d, (_, st) in zip(devs, scenes)]
        films = host.render_batch(items)
        for i, ((d, st), f) in enumerate(zip(items, films)):
            assert np.array_equal(_bits(f), _bits(d.render(st))), i
        host.close()
    finally:
        for d in devs:
            d.close()


def test_full_size_light_tracer(dev):
    s, st = procedural.cornell_box(800, 600)
    pst = st.replace(integrator=N.INTEGRATOR_PARTICLE, max_depth=-1, min_depth=7, seed=1)
    dev.upload(s)
    dev.set_counting(True)
    try:
        out = []
        for m in MODES:
            dev.set_renderer(m)
            out.append((dev.render_particles(pst, 1 << 22).astype(np.float64), dev.stats()))
    finally:
        dev.set_counting(False)
        dev.set_renderer(N.RENDERER_AUTO)
    want, cw = out[0]
    assert np.isfinite(want).all() and want.mean() > 0
    for m, (got, cg) in zip(MODES[1:], out[1:]):
        assert np.allclose(got, want, rtol=1e-5, atol=1e-6 * want.max()), m
        for k in ("rays_closest", "rays_shadow", "node_visits", "prim_tests"):
            assert cg[k] == cw[k], (m, k)
