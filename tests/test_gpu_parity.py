"""GPU parity: the CUDA library against the CPU oracle, through the C ABI.

The oracle restates the reference's algorithms on the same inputs (same scene,
same Philox streams, same deterministic math), so the expected agreement is
bit-for-bit: hit primitive ids, hit distances, barycentrics and tie flags of
ray batches, and every float of rendered films.
"""
import numpy as np
import pytest

from radiantium_gb300 import native as N
from radiantium_gb300 import procedural
from oracle.oracle import OracleScene, detmath

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def random_rays(scene_box, n, seed, inside=False):
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(scene_box[0], dtype=np.float64), np.asarray(scene_box[1], dtype=np.float64)
    ext = hi - lo
    rays = np.zeros(n, dtype=N.ray_dtype())
    if inside:
        o = lo + rng.random((n, 3)) * ext
    else:
        o = (lo + hi) / 2 + (rng.random((n, 3)) - 0.5) * ext * 3.0
    tgt = lo + rng.random((n, 3)) * ext
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["o"] = o.astype(np.float32)
    rays["d"] = d.astype(np.float32)
    rays["min_t"] = np.where(rng.random(n) < 0.5, 1e-4, 1.401298464324817e-45).astype(np.float32)
    rays["max_t"] = np.where(rng.random(n) < 0.8, 3.4028234663852886e38, rng.random(n) * 4).astype(np.float32)
    return rays


def assert_hits_equal(g, o):
    assert np.array_equal(g["prim"], o["prim"]), f"prim ids differ at {np.nonzero(g['prim'] != o['prim'])[0][:10]}"
    assert np.array_equal(g["sub"], o["sub"])
    assert np.array_equal(_bits(g["t"]), _bits(o["t"]))
    assert np.array_equal(_bits(g["u"]), _bits(o["u"]))
    assert np.array_equal(_bits(g["v"]), _bits(o["v"]))
    assert np.array_equal(g["flags"], o["flags"])


DM = {"sin": (0, 100, (-30, 30)), "cos": (1, 101, (-30, 30)), "tan": (2, 102, (-1.5, 1.5)),
      "atan": (3, 103, (-50, 50)), "atan2": (4, 104, (-3, 3)), "acos": (5, 105, (-1, 1)),
      "exp": (6, 106, (-90, 88)), "log": (7, 107, (1e-30, 1e30))}


@pytest.mark.parametrize("name", list(DM))
def test_detmath_device_matches_host_bitwise(dev, name):
    fn, cuda_fn, (lo, hi) = DM[name]
    rng = np.random.default_rng(fn)
    if name == "log":
        a = np.exp(rng.uniform(np.log(lo), np.log(hi), 200000)).astype(np.float32)
    else:
        a = rng.uniform(lo, hi, 200000).astype(np.float32)
    b = rng.uniform(-3, 3, 200000).astype(np.float32)
    gpu = dev.detmath(fn, a, b)
    host = detmath(name, a, b)
    assert np.array_equal(_bits(gpu), _bits(host)), name
    # and within 4 ulp of CUDA's own implementation
    ref = dev.detmath(cuda_fn, a, b)
    ok = np.isfinite(ref)
    ulp = np.abs(gpu[ok].astype(np.float64) - ref[ok]) / np.spacing(np.abs(ref[ok])).astype(np.float64)
    assert ulp.max() <= 4.0, (name, ulp.max())


@pytest.fixture(scope="module")
def cornell():
    s, st = procedural.cornell_box(64, 64)
    return s, st, OracleScene(s)


@pytest.fixture(scope="module")
def zoo():
    s, st = procedural.material_zoo(48, 48)
    return s, st, OracleScene(s)


def test_trace_closest_cornell(dev, cornell):
    s, st, orc = cornell
    dev.upload(s)
    rays = random_rays(((0, 0, 0), (1, 1, 1)), 100000, 1)
    rays = np.concatenate([rays, random_rays(((0, 0, 0), (1, 1, 1)), 50000, 2, inside=True)])
    assert_hits_equal(dev.trace_closest(rays), orc.trace_closest(rays))


def test_trace_any_cornell(dev, cornell):
    s, st, orc = cornell
    dev.upload(s)
    rays = random_rays(((0, 0, 0), (1, 1, 1)), 100000, 3, inside=True)
    assert np.array_equal(dev.trace_any(rays), orc.trace_any(rays))


def test_trace_instances_spheres(dev, zoo):
    s, st, orc = zoo
    dev.upload(s)
    rays = random_rays(((-3, 0, -2), (3, 3, 2)), 100000, 4)
    rays = np.concatenate([rays, random_rays(((-3, 0, -2), (3, 3, 2)), 50000, 5, inside=True)])
    g, o = dev.trace_closest(rays), orc.trace_closest(rays)
    assert_hits_equal(g, o)
    assert (o["sub"] >= 0).sum() > 100, "rays should hit instanced prototypes"
    assert np.array_equal(dev.trace_any(rays), orc.trace_any(rays))


def test_camera_rays_trace(dev, cornell):
    s, st, orc = cornell
    dev.upload(s)
    pos = np.random.default_rng(6).random((20000, 2)) * 64
    rays = orc.camera_rays(pos)
    assert_hits_equal(dev.trace_closest(rays), orc.trace_closest(rays))


RENDERERS = [N.RENDERER_MEGAKERNEL, N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH]


def _render(dev, st, renderer):
    dev.set_renderer(renderer)
    try:
        return dev.render(st)
    finally:
        dev.set_renderer(N.RENDERER_AUTO)


@pytest.mark.parametrize("renderer", RENDERERS)
@pytest.mark.parametrize("method", [N.METHOD_MIS, N.METHOD_NEE, N.METHOD_BXDF])
@pytest.mark.parametrize("strategy", [N.STRATEGY_UNIFORM, N.STRATEGY_ALL])
def test_render_cornell_bitexact(dev, cornell, method, strategy, renderer):
    s, st, orc = cornell
    dev.upload(s)
    st = st.replace(spp=3, method=method, strategy=strategy)
    g, o = _render(dev, st, renderer), orc.render(st)
    assert g.shape == (64, 64, 3)
    assert np.array_equal(_bits(g), _bits(o)), f"max abs diff {np.abs(g - o).max()}"


@pytest.mark.parametrize("renderer", RENDERERS)
@pytest.mark.parametrize("method", [N.METHOD_MIS, N.METHOD_NEE, N.METHOD_BXDF])
def test_render_materials_bitexact(dev, zoo, method, renderer):
    s, st, orc = zoo
    dev.upload(s)
    st = st.replace(method=method)
    g, o = _render(dev, st, renderer), orc.render(st)
    assert np.array_equal(_bits(g), _bits(o)), f"max abs diff {np.abs(g - o).max()}"


def test_wavefront_matches_megakernel_large(dev):
    """Many regenerated path slots: 96x96 x 16 spp of the instanced-sphere scene."""
    from radiantium_gb300 import procedural as P
    s, st = P.instanced_spheres(96, 96, sphere_n=12, grid=4, env_w=64, env_h=32)
    dev.upload(s)
    st = st.replace(spp=16)
    a = _render(dev, st, N.RENDERER_MEGAKERNEL)
    b = _render(dev, st, N.RENDERER_WAVEFRONT)
    assert np.array_equal(_bits(a), _bits(b)), f"max abs diff {np.abs(a - b).max()}"
    o = OracleScene(s).render(st.replace(x0=20, y0=30, width=24, height=16))
    assert np.array_equal(_bits(b[20:44, 30:46]), _bits(o))


def test_wavefront_tall_tree_matches_megakernel(dev):
    """A prototype of 12 * 64^2 = 49,152 triangles (one per leaf) has a tree of at
    least 17 levels, so the wavefront's trace kernels keep the bottom of their
    stacks in shared memory (trees of RT_DEEP_TREE = 16 levels or more): films and
    traversal counters equal the megakernel's for the host- and graph-driven loops."""
    from radiantium_gb300 import procedural as P
    s, st = P.instanced_spheres(64, 48, sphere_n=64, grid=2, env_w=64, env_h=32)
    dev.upload(s)
    st = st.replace(spp=8)
    dev.set_counting(True)
    try:
        a = _render(dev, st, N.RENDERER_MEGAKERNEL)
        ca = dev.stats()
        for mode in (N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH):
            b = _render(dev, st, mode)
            cb = dev.stats()
            assert np.array_equal(_bits(a), _bits(b)), (mode, float(np.abs(a - b).max()))
            if mode == N.RENDERER_WAVEFRONT:
                for k in ("samples", "rays_closest", "rays_shadow", "node_visits", "prim_tests", "instance_visits"):
                    assert ca[k] == cb[k], (k, ca[k], cb[k])
    finally:
        dev.set_counting(False)


@pytest.mark.parametrize("renderer", RENDERERS)
def test_render_volume_bitexact(dev, renderer):
    """vol_path: the megakernel for both light strategies, the wavefront (with its
    boundary walks traced as queued segments) for the Uniform strategy."""
    s, st = procedural.volume_box(40, 40)
    orc = OracleScene(s)
    dev.upload(s)
    for strategy in (N.STRATEGY_UNIFORM, N.STRATEGY_ALL):
        if renderer != N.RENDERER_MEGAKERNEL and strategy == N.STRATEGY_ALL:
            continue
        stx = st.replace(strategy=strategy)
        g, o = _render(dev, stx, renderer), orc.render(stx)
        assert np.array_equal(_bits(g), _bits(o)), f"max abs diff {np.abs(g - o).max()}"


def test_volume_wavefront_matches_megakernel_large(dev):
    """vol_path on the C3 geometry at reduced size: wavefront == megakernel, with
    several rounds and heavy slot reuse, and the counters of both agree."""
    s, st = procedural.volume_sphere(64, 64, sphere_n=24)
    dev.upload(s)
    stx = st.replace(spp=8, max_depth=12)
    dev.set_counting(True)
    a = _render(dev, stx, N.RENDERER_MEGAKERNEL)
    ca = dev.stats()
    b = _render(dev, stx, N.RENDERER_WAVEFRONT)
    cb = dev.stats()
    dev.set_counting(False)
    assert np.array_equal(_bits(a), _bits(b)), f"max abs diff {np.abs(a - b).max()}"
    for k in ("samples", "rays_closest", "node_visits", "prim_tests"):
        assert ca[k] == cb[k], (k, ca[k], cb[k])


def test_render_crop_and_resume(dev, cornell):
    """A crop renders the same pixels as the full film; sample_begin continues the streams."""
    s, st, orc = cornell
    dev.upload(s)
    full = dev.render(st.replace(spp=2))
    crop = dev.render(st.replace(spp=2, x0=10, y0=20, width=17, height=9))
    assert np.array_equal(_bits(crop), _bits(full[10:27, 20:29]))
    later = dev.render(st.replace(spp=2, sample_begin=2))
    assert np.array_equal(_bits(later), _bits(orc.render(st.replace(spp=2, sample_begin=2))))


@pytest.mark.parametrize("renderer", RENDERERS)
def test_counters_match_oracle(dev, cornell, renderer):
    s, st, orc = cornell
    dev.upload(s)
    dev.set_counting(True)
    st = st.replace(spp=2)
    _render(dev, st, renderer)
    g = dev.stats()
    dev.set_counting(False)
    _, o = orc.render(st, stats=True)
    for k in ("samples", "rays_closest", "rays_shadow", "node_visits", "prim_tests", "instance_visits"):
        assert g[k] == o[k], (k, g[k], o[k])


@pytest.mark.parametrize("renderer", [N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH])
@pytest.mark.parametrize("method", [N.METHOD_MIS, N.METHOD_NEE])
def test_all_light_strategy_on_the_wavefront(dev, zoo, method, renderer):
    """The All light strategy (PathTracer.cs:297-304) on the wavefront: every light
    of a vertex - the zoo's two quad triangles, its sphere emitter and its
    environment - is estimated in the reference's order, one light per
    iteration, before the continuation; films bit for bit and ray counts equal
    to the oracle's."""
    s, st, orc = zoo
    dev.upload(s)
    st = st.replace(method=method, strategy=N.STRATEGY_ALL, spp=2)
    dev.set_counting(True)
    try:
        g = _render(dev, st, renderer)
        gc = dev.stats()
    finally:
        dev.set_counting(False)
    o, oc = orc.render(st, stats=True)
    assert np.array_equal(_bits(g), _bits(o)), f"max abs diff {np.abs(g - o).max()}"
    if renderer == N.RENDERER_WAVEFRONT:
        for k in ("samples", "rays_closest", "rays_shadow", "node_visits", "prim_tests", "instance_visits"):
            assert gc[k] == oc[k], (k, gc[k], oc[k])


def test_vol_path_all_strategy_stays_on_the_megakernel(dev):
    s, st = procedural.volume_box(16, 16)
    dev.upload(s)
    st = st.replace(strategy=N.STRATEGY_ALL, spp=1)
    try:
        dev.set_renderer(N.RENDERER_WAVEFRONT)
        with pytest.raises(N.RTError) as e:
            dev.render(st)
        assert e.value.code == N.RT_ERR_UNSUPPORTED
        dev.set_renderer(N.RENDERER_AUTO)            # AUTO picks the megakernel
        assert np.array_equal(_bits(dev.render(st)), _bits(OracleScene(s).render(st)))
    finally:
        dev.set_renderer(N.RENDERER_AUTO)
