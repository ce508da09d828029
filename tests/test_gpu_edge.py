"""Edge cases through the C ABI against the oracle (gpu): scenes without lights
or without primitives, degenerate rays (zero or NaN direction, infinite or NaN
origin, empty or inverted [min_t, max_t]), empty ray batches, and depth limits
that end every path or particle before its first bounce."""
import numpy as np
import pytest

from radiantium_gb300 import native as N
from radiantium_gb300 import procedural
from radiantium_gb300.scene import Camera, Group, SceneDesc
from oracle.oracle import OracleScene

pytestmark = pytest.mark.gpu
RENDERERS = [N.RENDERER_MEGAKERNEL, N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH]


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _dark_cornell():
    s, st = procedural.cornell_box(32, 24)
    s.groups = [g for g in s.groups if not g.emissive]
    return s, st


def test_scene_without_lights(dev):
    """Scene.SampleLight has nothing to choose (pdf 0): every path and particle is black."""
    s, st = _dark_cornell()
    dev.upload(s)
    orc = OracleScene(s)
    try:
        want = orc.render(st.replace(spp=4))
        pst = st.replace(integrator=N.INTEGRATOR_PARTICLE)
        pwant = orc.render_particles(pst, 5000)
    finally:
        orc.close()
    assert not want.any() and not pwant.any()
    try:
        for mode in RENDERERS:
            dev.set_renderer(mode)
            assert np.array_equal(_bits(dev.render(st.replace(spp=4))), _bits(want)), mode
            assert np.array_equal(_bits(dev.render_particles(pst, 5000)), _bits(pwant)), mode
    finally:
        dev.set_renderer(N.RENDERER_AUTO)


def test_scene_without_primitives_is_rejected(dev):
    s = SceneDesc(camera=Camera.look_at(16, 16, 40.0, (0, 0, 3), (0, 0, 0)), name="env-only")
    s.groups.append(Group(N.GROUP_INFINITE_LIGHT, s.add_texture(procedural.gaussian_lobe_env(16, 8, 3))))
    with pytest.raises(N.RTError) as e:
        dev.upload(s)
    assert e.value.code == N.RT_ERR_INVALID_ARG
    with pytest.raises(ValueError):
        OracleScene(s)


def _degenerate_rays():
    nan, inf = np.nan, np.inf
    o = [(0.5, 0.5, 2), (0.5, 0.5, 2), (nan, 0, 0), (0.5, 0.5, 0.5), (inf, 0.5, 0.5), (0.5, 0.5, 2),
         (0.5, 0.5, 2), (0.5, 0.5, 0.5), (0.5, 0.5, 0.5), (-inf, -inf, -inf), (0.5, 0.5, 0.5), (0.5, 0.5, 2)]
    d = [(0, 0, 0), (0, 0, -1), (0, 0, -1), (nan, 1, 0), (-1, 0, 0), (0, 0, -1),
         (1e-30, 0, -1), (0, -1, 0), (0, 0, 1), (1, 1, 1), (inf, 0, 0), (-0.0, -0.0, -1)]
    lo = [1e-4, 1e-4, 1e-4, 1e-4, 1e-4, 5.0, 1e-4, 0.0, -1.0, 1e-4, 1e-4, 1e-4]
    hi = [1e30, 1e30, 1e30, 1e30, 1e30, 1.0, 1e30, 0.0, 1e30, inf, 1e30, nan]
    rays = np.zeros(len(o), dtype=N.ray_dtype())
    rays["o"], rays["d"] = np.array(o, np.float32), np.array(d, np.float32)
    rays["min_t"], rays["max_t"] = np.array(lo, np.float32), np.array(hi, np.float32)
    return rays


@pytest.mark.parametrize("name", ["cornell", "instanced"])
def test_degenerate_rays(dev, name):
    if name == "cornell":
        s, _ = procedural.cornell_box(32, 32)
    else:
        s, _ = procedural.instanced_spheres(32, 32, sphere_n=12, grid=4, env_w=32, env_h=16)
    rays = _degenerate_rays()
    dev.upload(s)
    orc = OracleScene(s)
    try:
        want_h, want_a = orc.trace_closest(rays), orc.trace_any(rays)
    finally:
        orc.close()
    got_h, got_a = dev.trace_closest(rays), dev.trace_any(rays)
    for k in ("prim", "sub", "flags"):
        assert np.array_equal(got_h[k], want_h[k]), k
    for k in ("t", "u", "v"):
        assert np.array_equal(_bits(got_h[k]), _bits(want_h[k])), k
    assert np.array_equal(got_a.astype(np.uint8), want_a.astype(np.uint8))


@pytest.mark.parametrize("name", ["cornell", "instanced", "zoo"])
def test_axis_parallel_rays_match_oracle(dev, name):
    """200 k rays with exactly-zero direction components (along the axes and in
    the coordinate planes, signed zeros included): 1/d is infinite, and the
    slab test's IEEE semantics (BoundingBox3F.cs:155-176; 0 * inf is NaN, which
    its comparisons ignore) decide which boxes are entered.  Hits, tie flags
    and traversal counters equal the oracle's."""
    from tests.test_gpu_wide_traversal import _axis_rays
    if name == "cornell":
        s, _ = procedural.cornell_box(32, 32)
    elif name == "zoo":
        s, _ = procedural.material_zoo(32, 32)
    else:
        s, _ = procedural.instanced_spheres(32, 32, sphere_n=12, grid=4, env_w=32, env_h=16)
    rays = _axis_rays(s, 200000, 17)
    dev.upload(s)
    orc = OracleScene(s)
    try:
        want_h, want_hc = orc.trace_closest(rays, stats=True)
        want_a, want_ac = orc.trace_any(rays, stats=True)
    finally:
        orc.close()
    dev.set_counting(True)
    try:
        got_h = dev.trace_closest(rays)
        got_hc = dev.stats()
        got_a = dev.trace_any(rays)
        got_ac = dev.stats()
    finally:
        dev.set_counting(False)
    for k in ("prim", "sub", "flags"):
        assert np.array_equal(got_h[k], want_h[k]), k
    for k in ("t", "u", "v"):
        assert np.array_equal(_bits(got_h[k]), _bits(want_h[k])), k
    assert np.array_equal(got_a.astype(np.uint8), want_a.astype(np.uint8))
    for k in ("node_visits", "prim_tests", "instance_visits"):
        assert got_hc[k] == want_hc[k], ("closest", k, got_hc[k], want_hc[k])
        assert got_ac[k] == want_ac[k], ("any", k, got_ac[k], want_ac[k])
    assert (want_h["prim"] >= 0).sum() > rays.size // 10


def test_empty_ray_batch(dev):
    s, _ = procedural.cornell_box(16, 16)
    dev.upload(s)
    rays = np.zeros(0, dtype=N.ray_dtype())
    assert dev.trace_closest(rays).shape == (0,)
    assert dev.trace_any(rays).shape == (0,)


@pytest.mark.parametrize("max_depth", [0, 1])
def test_depth_limit_before_the_first_bounce(dev, max_depth):
    """path: max_depth 0 keeps only what the camera ray sees directly (no NEE) for the
    Bxdf method; the light tracer with max_depth 1 traces no particle ray, so its film
    is exactly CameraTraceLight (no float atomics involved)."""
    s, st = procedural.cornell_box(32, 24)
    dev.upload(s)
    orc = OracleScene(s)
    try:
        pst = st.replace(integrator=N.INTEGRATOR_PARTICLE, max_depth=max_depth)
        pwant = orc.render_particles(pst, 3000)
        cst = st.replace(spp=2, max_depth=max_depth, method=N.METHOD_BXDF)
        want = orc.render(cst)
    finally:
        orc.close()
    try:
        for mode in RENDERERS:
            dev.set_renderer(mode)
            assert np.array_equal(_bits(dev.render(cst)), _bits(want)), mode
            assert np.array_equal(_bits(dev.render_particles(pst, 3000)), _bits(pwant)), mode
    finally:
        dev.set_renderer(N.RENDERER_AUTO)


def test_h2d_byte_counts(dev):
    """rt_stats.h2d_bytes counts what a call copies from host memory to the device: a host ray
    batch exactly its rays, the megakernel nothing (its parameters are kernel arguments), a
    wavefront render its job table and queue counters (a few hundred bytes per round)."""
    s, st = procedural.cornell_box(32, 24)
    dev.upload(s)
    rays = np.zeros(100, dtype=N.ray_dtype())
    rays["o"][:] = (0.0, 0.5, 0.0)
    rays["d"][:] = (0.0, 0.0, 1.0)
    rays["min_t"], rays["max_t"] = 1e-4, 1e30
    dev.trace_closest(rays)
    assert dev.stats()["h2d_bytes"] == rays.nbytes
    dev.trace_any(rays)
    assert dev.stats()["h2d_bytes"] == rays.nbytes
    try:
        dev.set_renderer(N.RENDERER_MEGAKERNEL)
        dev.render(st.replace(spp=2))
        assert dev.stats()["h2d_bytes"] == 0
        for m in (N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH):
            dev.set_renderer(m)
            dev.render(st.replace(spp=2))
            assert 0 < dev.stats()["h2d_bytes"] < 1 << 16, m
            dev.render_particles(st.replace(integrator=N.INTEGRATOR_PARTICLE), 5000)
            assert 0 < dev.stats()["h2d_bytes"] < 1 << 16, m
    finally:
        dev.set_renderer(N.RENDERER_AUTO)
