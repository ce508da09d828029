"""The light tracer ("adjoint_particle": AdjointParticleIntegrator +
AdjointParticleRenderer) on the GPU against the oracle (gpu).

Each particle's camera connections (pixel and colour of every splat) must
equal the oracle's bit for bit: the particle's random stream, emission,
bounces, importance-mode BSDFs, camera sampling and visibility tests are
deterministic.  The film is the sum of those splats, added on the GPU with
float atomics in no fixed order (as under the reference's lock), so films
are compared within a summation-order tolerance: every splat is positive, so
the relative error of a pixel is below (splats in it) x 2^-24; the tests
allow 1e-5 relative plus 1e-6 of the image maximum.  The finishing pass
(scale by ScreenX * ScreenY / N plus CameraTraceLight) is the same arithmetic
on both sides.
"""
import ctypes as C

import numpy as np
import pytest

from radiantium_gb300 import native as N
from radiantium_gb300 import procedural
from oracle import oracle

pytestmark = pytest.mark.gpu
RTOL, ATOL_REL = 1e-5, 1e-6


def _particle(st, **kw):
    return st.replace(integrator=N.INTEGRATOR_PARTICLE, **kw)


SCENES = {
    "cornell": lambda: procedural.cornell_box(64, 48),
    "zoo": lambda: procedural.material_zoo(40, 32),
    "instanced": lambda: procedural.instanced_spheres(48, 32, sphere_n=12, grid=4, env_w=64, env_h=32),
    "volume": lambda: procedural.volume_box(32, 24),
}


def _set_limits(dev, sample_budget, capacity):
    f = dev.lib.rt_debug_set_limits
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_int64, C.c_int]
    assert f(dev.h, sample_budget, capacity) == N.RT_OK


def _film_close(got, want):
    tol = RTOL * np.abs(want) + ATOL_REL * float(np.abs(want).max())
    bad = np.abs(got.astype(np.float64) - want) > tol
    return int(bad.sum())


@pytest.mark.parametrize("name", list(SCENES))
@pytest.mark.parametrize("depth", [(-1, 3, 0.99), (4, 1, 0.7), (2, 0, 0.99)], ids=["unbounded", "d4", "d2"])
def test_splats_match_oracle(dev, name, depth):
    s, st = SCENES[name]()
    pst = _particle(st, max_depth=depth[0], min_depth=depth[1], rr_threshold=depth[2], seed=21)
    dev.upload(s)
    orc = oracle.OracleScene(s)
    try:
        n0, pix0, rgb0 = orc.particle_splats(pst, 4096, 16, first=123456789)
    finally:
        orc.close()
    n1, pix1, rgb1 = dev.particle_splats(pst, 4096, 16, first=123456789)
    assert n0.sum() > 100
    assert np.array_equal(n1, n0)
    assert np.array_equal(pix1, pix0)
    assert np.array_equal(rgb1.view(np.uint32), rgb0.view(np.uint32))


def test_particle_streams_above_2_32(dev):
    """Particle indices past 2^32 use the counter's second word."""
    s, st = SCENES["cornell"]()
    pst = _particle(st, max_depth=-1, seed=3)
    dev.upload(s)
    orc = oracle.OracleScene(s)
    try:
        want = orc.particle_splats(pst, 1024, 8, first=(1 << 32) - 512)
    finally:
        orc.close()
    got = dev.particle_splats(pst, 1024, 8, first=(1 << 32) - 512)
    for a, b in zip(got, want):
        assert np.array_equal(a.view(np.uint32) if a.dtype == np.float32 else a,
                              b.view(np.uint32) if b.dtype == np.float32 else b)


RENDERERS = [N.RENDERER_MEGAKERNEL, N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH]


@pytest.mark.parametrize("name", ["cornell", "zoo", "instanced", "volume"])
def test_film_matches_oracle(dev, name):
    """Every renderer's film within the summation tolerance, and exactly the
    oracle's ray, node, primitive and instance counts (the same rays traced)."""
    s, st = SCENES[name]()
    pst = _particle(st, seed=9)
    dev.upload(s)
    orc = oracle.OracleScene(s)
    try:
        want, ost = orc.render_particles(pst, 200000, stats=True)
    finally:
        orc.close()
    assert np.isfinite(want).all()
    dev.set_counting(True)
    try:
        for mode in RENDERERS:
            dev.set_renderer(mode)
            got = dev.render_particles(pst, 200000)
            gst = dev.stats()
            assert _film_close(got, want) == 0, mode
            assert gst["samples"] == 200000
            for k in ("rays_closest", "rays_shadow", "node_visits", "prim_tests", "instance_visits"):
                assert gst[k] == ost[k], (mode, k)
    finally:
        dev.set_counting(False)
        dev.set_renderer(N.RENDERER_AUTO)


def test_wavefront_small_slot_pool(dev):
    """Far more particles than path slots: slots are refilled until the range is done."""
    s, st = SCENES["zoo"]()
    pst = _particle(st, seed=13, max_depth=-1, min_depth=5)
    dev.upload(s)
    dev.set_renderer(N.RENDERER_MEGAKERNEL)
    try:
        want = dev.render_particles(pst, 50000).astype(np.float64)
        dev.set_renderer(N.RENDERER_WAVEFRONT)
        _set_limits(dev, 1 << 24, 1000)
        got = dev.render_particles(pst, 50000)
    finally:
        _set_limits(dev, 1 << 24, N.MAX_SLOTS)
        dev.set_renderer(N.RENDERER_AUTO)
    assert _film_close(got, want) == 0


@pytest.mark.parametrize("mode", [N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH])
def test_wavefront_rounds(dev, mode):
    """A particle range longer than one round (4 x the sample budget) renders in
    rounds; the film is the same as the megakernel's."""
    s, st = SCENES["instanced"]()
    pst = _particle(st, seed=17)
    dev.upload(s)
    dev.set_renderer(N.RENDERER_MEGAKERNEL)
    try:
        want = dev.render_particles(pst, 30000, first=77).astype(np.float64)
        dev.set_renderer(mode)
        _set_limits(dev, 1000, 0)          # rounds of 4000 particles
        got = dev.render_particles(pst, 30000, first=77)
    finally:
        _set_limits(dev, 1 << 24, 0)
        dev.set_renderer(N.RENDERER_AUTO)
    assert _film_close(got, want) == 0


def test_tall_tree_wavefront_matches_megakernel(dev):
    """A 49,152-triangle prototype (trees of 17+ levels: the shared-memory stack
    trace kernels): the wavefront traces the megakernel's rays and node visits."""
    s, st = procedural.instanced_spheres(48, 32, sphere_n=64, grid=2, env_w=64, env_h=32)
    pst = _particle(st, seed=23)
    dev.upload(s)
    dev.set_counting(True)
    try:
        dev.set_renderer(N.RENDERER_MEGAKERNEL)
        want = dev.render_particles(pst, 100000).astype(np.float64)
        cw = dev.stats()
        for mode in (N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH):
            dev.set_renderer(mode)
            got = dev.render_particles(pst, 100000)
            cg = dev.stats()
            assert _film_close(got, want) == 0, mode
            for k in ("rays_closest", "rays_shadow", "node_visits", "prim_tests", "instance_visits"):
                assert cg[k] == cw[k], (mode, k)
    finally:
        dev.set_counting(False)
        dev.set_renderer(N.RENDERER_AUTO)


def test_golden_particles(dev):
    """Against the committed fixtures (made by the oracle; this test reads them as files)."""
    import os
    from tests.golden import make_golden
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    for name, s, st in make_golden.particle_cases():
        with np.load(os.path.join(here, f"particles_{name}.npz")) as z:
            g = {k: z[k] for k in z.files}
        pst = _particle(st, seed=5)
        dev.upload(s)
        n, pix, rgb = dev.particle_splats(pst, 512, 12, first=1000)
        assert np.array_equal(n, g["n"]), name
        assert np.array_equal(pix, g["pix"]), name
        assert np.array_equal(rgb.view(np.uint32), g["rgb"]), name
        film = dev.render_particles(pst, 20000)
        assert _film_close(film, g["film"].view(np.float32).astype(np.float64)) == 0, name


def test_ranges_combine(dev):
    """Films of disjoint particle ranges average (weighted by count) to the film of their union."""
    s, st = SCENES["cornell"]()
    pst = _particle(st, seed=4)
    dev.upload(s)
    whole = dev.render_particles(pst, 300000).astype(np.float64)
    a = dev.render_particles(pst, 100000, first=0).astype(np.float64)
    b = dev.render_particles(pst, 200000, first=100000).astype(np.float64)
    # CameraTraceLight is in every film once, so it survives the weighted mean unchanged
    mix = (a * 100000 + b * 200000) / 300000
    assert np.allclose(mix, whole, rtol=1e-4, atol=1e-5 * whole.max())


def test_device_output_equals_host(dev):
    torch = pytest.importorskip("torch")
    s, st = SCENES["cornell"]()
    pst = _particle(st, seed=8)
    dev.upload(s)
    host = dev.render_particles(pst, 4096)
    out = torch.zeros(s.camera.width * s.camera.height * 3, dtype=torch.float32, device="cuda")
    dev.render_particles_device(pst, 4096, out.data_ptr())
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(host.shape)
    assert _film_close(got, host.astype(np.float64)) == 0


def test_errors(dev):
    s, st = SCENES["cornell"]()
    dev.upload(s)
    pst = _particle(st)
    for bad, kw in ((st, {}), (pst.replace(x0=1), {}), (pst, {"count": 0}), (pst, {"first": -1})):
        with pytest.raises(N.RTError) as e:
            dev.render_particles(bad, kw.get("count", 16), first=kw.get("first", 0))
        assert e.value.code == N.RT_ERR_INVALID_ARG
    with pytest.raises(N.RTError) as e:
        dev.render(pst)
    assert e.value.code == N.RT_ERR_INVALID_ARG


def test_scene_file_particle_renderer(tmp_path):
    """A reference-schema scene file with the adjoint_particle integrator, rendered through
    GpuRenderer (16 passes of particle ranges, count-weighted mean) against the oracle."""
    from radiantium_gb300.config import load_scene_file
    from tests.test_cpu_config import _scene_file
    r = load_scene_file(_scene_file(tmp_path, {"type": "adjoint_particle", "min_depth": 4},
                                    {"particle_count": 160000}))
    r.Start()
    r.Wait()
    assert r.IsSuccess and r.CompletedTaskCount == 16
    orc = oracle.OracleScene(r.scene)
    try:
        want = orc.render_particles(r.settings, 160000)
    finally:
        orc.close()
    got = r.RenderTarget.astype(np.float64)
    assert np.allclose(got, want, rtol=1e-4, atol=1e-5 * float(np.abs(want).max()))
