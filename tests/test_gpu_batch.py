"""Batched rendering (rt_render_batch) against one-scene renders (gpu).

A batch renders several scenes in one wavefront.  Every film must equal the
film rt_render gives for the same item, bit for bit: a sample's random
stream and its pixel's summation order do not depend on what else is in
flight.  Checked with the bounce loop as a CUDA graph and driven from the
host, and with sample rounds and heavy path-slot reuse forced by small
limits.
"""
import ctypes as C

import numpy as np
import pytest

from radiantium_gb300 import native as N
from radiantium_gb300 import procedural
from radiantium_gb300.device import Device

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _set_limits(dev, sample_budget, capacity):
    f = dev.lib.rt_debug_set_limits
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int64, C.c_int]
    assert f(dev.h, sample_budget, capacity) == N.RT_OK


@pytest.fixture(scope="module")
def scenes():
    specs = [procedural.cornell_box(48, 40), procedural.material_zoo(40, 32),
             procedural.instanced_spheres(64, 48, sphere_n=8, grid=3, env_w=32, env_h=16)]
    devs = []
    for s, st in specs:
        d = Device(0)
        d.upload(s)
        devs.append((d, st))
    yield devs
    for d, _ in devs:
        d.close()


def _items(devs):
    (a, sa), (b, sb), (c, sc) = devs
    return [(a, sa.replace(spp=5, seed=3)),
            (b, sb.replace(spp=3, seed=4, method=N.METHOD_NEE)),
            (c, sc.replace(spp=4, seed=5, x0=8, y0=6, width=40, height=30)),
            (a, sa.replace(spp=2, seed=9, method=N.METHOD_BXDF))]


def _singles(items):
    out = []
    for d, st in items:
        d.set_renderer(N.RENDERER_MEGAKERNEL)
        out.append(d.render(st))
        d.set_renderer(N.RENDERER_AUTO)
    return out


@pytest.mark.parametrize("mode", [N.RENDERER_WAVEFRONT_GRAPH, N.RENDERER_WAVEFRONT])
@pytest.mark.parametrize("limits", [(0, 0), (3000, 512)])
def test_batch_matches_single_renders(scenes, mode, limits):
    items = _items(scenes)
    want = _singles(items)
    host = Device(0)
    try:
        if limits != (0, 0):
            _set_limits(host, *limits)
        host.set_renderer(mode)
        got = host.render_batch(items)
        for i, (g, w) in enumerate(zip(got, want)):
            assert g.shape == w.shape
            assert np.array_equal(_bits(g), _bits(w)), f"item {i}: max abs diff {np.abs(g - w).max()}"
        st = host.stats()
        assert st["samples"] == sum(g.shape[0] * g.shape[1] * it[1].spp for g, it in zip(got, items))
    finally:
        host.close()


def test_batch_repeats_and_single_graph_render(scenes):
    """Two batches in a row on one context (the graph is reused), and the
    one-scene graph renderer with several rounds, against the megakernel."""
    items = _items(scenes)
    want = _singles(items)
    host = Device(0)
    try:
        host.set_renderer(N.RENDERER_WAVEFRONT_GRAPH)
        for _ in range(2):
            got = host.render_batch(items)
            for g, w in zip(got, want):
                assert np.array_equal(_bits(g), _bits(w))
    finally:
        host.close()
    d, st = scenes[2]
    _set_limits(d, 2000, 300)
    d.set_renderer(N.RENDERER_WAVEFRONT_GRAPH)
    try:
        g = d.render(st.replace(spp=3, seed=21))
    finally:
        d.set_renderer(N.RENDERER_MEGAKERNEL)
    w = d.render(st.replace(spp=3, seed=21))
    d.set_renderer(N.RENDERER_AUTO)
    _set_limits(d, 1 << 24, N.MAX_SLOTS)
    assert np.array_equal(_bits(g), _bits(w))


def test_batch_of_volumes_matches_single_renders():
    vols = [procedural.volume_box(40, 40, seed=s) for s in (9, 10)]
    devs = []
    try:
        for s, st in vols:
            d = Device(0)
            d.upload(s)
            devs.append((d, st))
        items = [(devs[0][0], devs[0][1].replace(spp=3, seed=2)), (devs[1][0], devs[1][1].replace(spp=5, seed=3)),
                 (devs[0][0], devs[0][1].replace(spp=2, seed=4, x0=5, y0=7, width=20, height=16))]
        want = _singles(items)
        host = Device(0)
        try:
            _set_limits(host, 2500, 256)
            got = host.render_batch(items)
            for g, w in zip(got, want):
                assert np.array_equal(_bits(g), _bits(w))
        finally:
            host.close()
    finally:
        for d, _ in devs:
            d.close()


def test_batch_all_light_strategy(scenes):
    """`path` items with the All light strategy (every light estimated at each
    vertex, one light per wavefront iteration) reproduce their single renders,
    Uniform items alongside them too."""
    (a, sa), (b, sb), _ = scenes
    host = Device(0)
    try:
        items = [(a, sa.replace(spp=2, strategy=N.STRATEGY_ALL)), (b, sb.replace(spp=2)),
                 (b, sb.replace(spp=1, seed=9, strategy=N.STRATEGY_ALL))]
        films = host.render_batch(items)
        for (d, st), f in zip(items, films):
            assert np.array_equal(_bits(f), _bits(d.render(st)))
    finally:
        host.close()


def test_batch_rejects_unsupported_items(scenes):
    (a, sa), (b, sb), _ = scenes
    host = Device(0)
    try:
        with pytest.raises(N.RTError) as e:
            host.render_batch([(a, sa.replace(spp=1)), (b, sb.replace(spp=1, integrator=N.INTEGRATOR_VOL_PATH))])
        assert e.value.code == N.RT_ERR_UNSUPPORTED
        with pytest.raises(N.RTError) as e:
            host.render_batch([(a, sa.replace(spp=1, integrator=N.INTEGRATOR_VOL_PATH, strategy=N.STRATEGY_ALL))])
        assert e.value.code == N.RT_ERR_UNSUPPORTED
        with pytest.raises(N.RTError) as e:
            host.render_batch([(a, sa.replace(spp=1))] * (N.MAX_BATCH + 1))
        assert e.value.code == N.RT_ERR_INVALID_ARG
    finally:
        host.close()


def test_autotune_keeps_films(scenes):
    """rt_autotune only picks settings that leave films unchanged: a batch
    rendered after tuning equals the one-scene megakernel renders."""
    items = _items(scenes)
    want = _singles(items)
    host = Device(0)
    try:
        r = host.autotune([(d, st.replace(spp=1)) for d, st in items])
        assert r["capacity"] in (N.MAX_SLOTS, N.MAX_SLOTS // 2, N.MAX_SLOTS // 4)
        assert r["refill"] in (4, 8, 16)
        assert r["renderer"] in (N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH)
        assert 0 < r["ms"] <= r["ms_default"]
        got = host.render_batch(items)
        for g, w in zip(got, want):
            assert np.array_equal(_bits(g), _bits(w))
    finally:
        host.close()
