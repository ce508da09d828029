"""Gradients of the MIS path tracer (rt_adjoint_*) against central finite
differences of the renderer itself (gpu).

The loss is linearised at the parameters: l(theta) = sum(w * I(theta)) with
fixed pixel weights w = dL/dI of an L2 loss against a target film rendered
with perturbed parameters.  Finite differences use common random numbers
(the same seed at theta + eps v and theta - eps v):
  - albedo: the film is linear in the albedo texels along a fixed path, so
    the adjoint equals the finite difference up to float rounding (1 %);
  - alpha: GGX sampling moves with alpha, so finite differences carry
    visibility-change noise; checked along a high-signal direction (sign of
    the gradient, steps relative to each alpha) against the mean of 16
    seeds x 16384 spp, within 2 % (the standard error of that mean is
    about 1.2 %).
These run on a reduced scene (48 x 48, 10,800 triangles, 32 x 32 texture).  At
the benchmark configuration (256 x 256, 64 spp, depth 6, 199,692 triangles,
512 x 512 texture) the alpha gradient is checked material by material for the
four largest components and along a random direction, and the finite
differences are shown to be those of the oracle's restatement of the
reference's renderer: its films at the perturbed parameters equal the GPU's
bit for bit.
"""
import math

import numpy as np
import pytest

from radiantium_gb300 import native as N
from radiantium_gb300 import procedural
from radiantium_gb300.device import Device

pytestmark = pytest.mark.gpu

ALBEDO_TOL = 0.01
ALPHA_TOL = 0.02


@pytest.fixture(scope="module")
def adj():
    s, st, prm = procedural.adjoint_patches(48, 48, sphere_n=30, tex_size=32)
    d = Device(0)
    d.upload(s)
    rng = np.random.default_rng(0)
    ti, rts, alpha0 = prm["albedo_texture"], prm["roughness_textures"], prm["alpha"].copy()
    alb0 = s.textures[ti].data.copy()

    def set_params(alb, alpha):
        d.update_texture(ti, alb)
        for t, a in zip(rts, alpha):
            d.update_texture(t, np.full(3, math.sqrt(a), np.float32))

    set_params(np.clip(alb0 * rng.uniform(0.7, 1.3, alb0.shape), 0.05, 0.95).astype(np.float32),
               alpha0 * rng.uniform(0.7, 1.3, alpha0.shape))
    target = d.render(st.replace(spp=4096, seed=99))
    set_params(alb0, alpha0)
    ref = d.render(st.replace(spp=4096, seed=77))
    w = (2 * (ref - target)).astype(np.float32)
    yield d, st, prm, alb0, alpha0, w, set_params
    set_params(alb0, alpha0)
    d.close()


def _lin(d, st, w):
    return float((w.astype(np.float64) * d.render(st)).sum())


def test_forward_is_the_render(adj):
    d, st, *_ = adj
    stx = st.replace(spp=8, seed=5)
    a, b = d.adjoint_forward(stx), d.render(stx)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_backward_counts_its_host_copies(adj):
    """rt_stats.h2d_bytes of the backward pass: dL/dI (w * h * 3 floats) plus its small tables."""
    d, st, prm, _, _, w, _ = adj
    d.adjoint_backward(st.replace(spp=2, seed=4), w, prm["albedo_texture"], prm["alpha_materials"])
    h = d.stats()["h2d_bytes"]
    assert w.size * 4 < h < w.size * 4 + (1 << 16)


def test_albedo_gradient_matches_fd(adj):
    d, st, prm, alb0, alpha0, w, set_params = adj
    stx = st.replace(spp=256, seed=3)
    g, _ = d.adjoint_backward(stx, w, prm["albedo_texture"], [])
    g = g.reshape(-1).astype(np.float64)
    rng = np.random.default_rng(1)
    v = rng.standard_normal(alb0.shape).astype(np.float32)
    eps = 1e-3
    set_params(alb0 + eps * v, alpha0)
    lp = _lin(d, stx, w)
    set_params(alb0 - eps * v, alpha0)
    lm = _lin(d, stx, w)
    set_params(alb0, alpha0)
    fd, ad = (lp - lm) / (2 * eps), float((g * v).sum())
    assert abs(fd - ad) <= ALBEDO_TOL * abs(fd), (fd, ad)
    # the texels with the largest gradients, one at a time
    for i in np.argsort(-np.abs(g))[:4]:
        e = np.zeros_like(alb0)
        e[i] = 1e-2
        set_params(alb0 + e, alpha0)
        lp = _lin(d, stx, w)
        set_params(alb0 - e, alpha0)
        lm = _lin(d, stx, w)
        set_params(alb0, alpha0)
        fd = (lp - lm) / 2e-2
        assert abs(fd - g[i]) <= ALBEDO_TOL * abs(fd) + 1e-7, (i, fd, g[i])


def test_alias_light_sampling_replays_the_same_paths(adj):
    """With alias-table env sampling the replay draws the same texels as the
    forward pass: the forward film is the alias-mode render, and the albedo
    gradient matches finite differences of alias-mode renders."""
    d, st, prm, alb0, alpha0, w, set_params = adj
    d.set_light_sampling(N.LIGHT_SAMPLING_ALIAS)
    try:
        stx = st.replace(spp=256, seed=3)
        a = d.adjoint_forward(stx)
        assert np.array_equal(a.view(np.uint32), d.render(stx).view(np.uint32))
        d.set_light_sampling(N.LIGHT_SAMPLING_CDF)
        assert not np.array_equal(a.view(np.uint32), d.render(stx).view(np.uint32))
        d.set_light_sampling(N.LIGHT_SAMPLING_ALIAS)
        g, _ = d.adjoint_backward(stx, w, prm["albedo_texture"], [])
        g = g.reshape(-1).astype(np.float64)
        v = np.random.default_rng(2).standard_normal(alb0.shape).astype(np.float32)
        eps = 1e-3
        set_params(alb0 + eps * v, alpha0)
        lp = _lin(d, stx, w)
        set_params(alb0 - eps * v, alpha0)
        lm = _lin(d, stx, w)
        set_params(alb0, alpha0)
        fd, ad = (lp - lm) / (2 * eps), float((g * v).sum())
        assert abs(fd - ad) <= ALBEDO_TOL * abs(fd), (fd, ad)
    finally:
        d.set_light_sampling(N.LIGHT_SAMPLING_CDF)
        set_params(alb0, alpha0)


def test_alpha_gradient_matches_fd(adj):
    d, st, prm, alb0, alpha0, w, set_params = adj
    _, g = d.adjoint_backward(st.replace(spp=65536, seed=8), w, -1, prm["alpha_materials"])
    v = np.sign(g) * alpha0
    ad = float((g.astype(np.float64) * v).sum())
    eps, fds = 0.01, []
    for seed in range(16):
        stx = st.replace(spp=16384, seed=100 + seed)
        set_params(alb0, alpha0 + eps * v)
        lp = _lin(d, stx, w)
        set_params(alb0, alpha0 - eps * v)
        lm = _lin(d, stx, w)
        fds.append((lp - lm) / (2 * eps))
    set_params(alb0, alpha0)
    fd = float(np.mean(fds))
    assert abs(fd - ad) <= ALPHA_TOL * abs(fd), (fd, ad, fds)


def test_update_texture_and_errors(adj):
    d, st, prm, alb0, alpha0, w, set_params = adj
    stx = st.replace(spp=4, seed=5)
    base = d.render(stx)
    d.update_texture(prm["albedo_texture"], alb0 * 0.5)
    half = d.render(stx)
    d.update_texture(prm["albedo_texture"], alb0)
    assert np.array_equal(d.render(stx).view(np.uint32), base.view(np.uint32))
    assert not np.array_equal(half, base)
    env = len(d.scene.textures) - 1
    with pytest.raises(N.RTError) as e:
        d.update_texture(env, d.scene.textures[env].data)
    assert e.value.code == N.RT_ERR_UNSUPPORTED
    with pytest.raises(N.RTError) as e:
        d.adjoint_backward(stx.replace(method=N.METHOD_NEE), w, prm["albedo_texture"], [])
    assert e.value.code == N.RT_ERR_UNSUPPORTED
    m = prm["alpha_materials"][0]
    with pytest.raises(N.RTError) as e:
        d.adjoint_backward(stx, w, -1, [m, m])
    assert e.value.code == N.RT_ERR_INVALID_ARG


def test_albedo_gradient_all_lights_path(adj):
    """The All light strategy runs the megakernel adjoint (two passes per
    sample in one thread): same finite-difference check."""
    d, st, prm, alb0, alpha0, w, set_params = adj
    stx = st.replace(spp=64, seed=4, strategy=N.STRATEGY_ALL)
    g, _ = d.adjoint_backward(stx, w, prm["albedo_texture"], [])
    rng = np.random.default_rng(2)
    v = rng.standard_normal(alb0.shape).astype(np.float32)
    eps = 1e-3
    set_params(alb0 + eps * v, alpha0)
    lp = _lin(d, stx, w)
    set_params(alb0 - eps * v, alpha0)
    lm = _lin(d, stx, w)
    set_params(alb0, alpha0)
    fd, ad = (lp - lm) / (2 * eps), float((g.reshape(-1).astype(np.float64) * v).sum())
    assert abs(fd - ad) <= ALBEDO_TOL * abs(fd), (fd, ad)


# ---- the C5 configuration: 256 x 256, 64 spp, depth 6, 199,692 triangles, 512 x 512 albedo texture ----
C5_FD_SEEDS, C5_FD_SPP = 6, 4096


@pytest.fixture(scope="module")
def c5():
    """The adjoint benchmark's scene, parameters and loss weights (bench.adjoint_setup)."""
    import bench
    s, st, prm = procedural.adjoint_patches()
    d = Device(0)
    d.upload(s)
    alb0, alpha0, set_params, (alb_t, alpha_t) = bench.adjoint_setup(d, prm)
    set_params(alb_t, alpha_t)
    target = d.render(st.replace(spp=256, seed=99))
    set_params(alb0, alpha0)
    ref = d.render(st.replace(spp=1024, seed=77))
    w = (2 * (ref - target)).astype(np.float32)
    yield d, s, st, prm, alb0, alpha0, w, set_params
    set_params(alb0, alpha0)
    d.close()


def _fd(d, st, w, set_params, alb0, alpha0, v, eps):
    """Central differences of the linearised loss along alpha direction v, common
    random numbers per seed: (mean, standard error of the mean)."""
    fds = []
    for k in range(C5_FD_SEEDS):
        stx = st.replace(spp=C5_FD_SPP, seed=100 + k)
        set_params(alb0, alpha0 + eps * v)
        lp = _lin(d, stx, w)
        set_params(alb0, alpha0 - eps * v)
        lm = _lin(d, stx, w)
        fds.append((lp - lm) / (2 * eps))
    set_params(alb0, alpha0)
    return float(np.mean(fds)), float(np.std(fds, ddof=1) / math.sqrt(len(fds)))


def test_c5_alpha_gradient_per_material(c5):
    """At the benchmark configuration: the alpha gradient of each of the 4
    materials with the largest |dL/dalpha| (one material at a time, steps of 5 %
    of its alpha) and along one random direction over all 64 alphas (2 % steps),
    against central differences of the renderer (6 seeds x 4096 spp, common
    random numbers).  Bound: 2 % of the finite difference plus 3 standard errors
    of its seed mean (visibility changes make finite differences of alpha noisy;
    the adjoint at 16384 spp is far less so)."""
    d, s, st, prm, alb0, alpha0, w, set_params = c5
    _, g = d.adjoint_backward(st.replace(spp=16384, seed=8), w, -1, prm["alpha_materials"])
    g = g.astype(np.float64)
    top = np.argsort(-np.abs(g))[:4]
    dirs = [(f"material {m}", np.eye(alpha0.size)[m] * alpha0[m], 0.05) for m in top]
    dirs.append(("random", np.random.default_rng(5).standard_normal(alpha0.size) * alpha0, 0.02))
    report = []
    for name, v, eps in dirs:
        fd, se = _fd(d, st, w, set_params, alb0, alpha0, v, eps)
        ad = float((g * v).sum())
        report.append((name, fd, se, ad))
        assert abs(fd - ad) <= ALPHA_TOL * abs(fd) + 3 * se, (name, fd, se, ad, report)
    # the well-determined ones (standard error under 1.5 %) meet 2 % on their own
    sharp = [r for r in report if r[2] < 0.015 * abs(r[1])]
    assert len(sharp) >= 2, report
    for name, fd, se, ad in sharp:
        assert abs(fd - ad) <= ALPHA_TOL * abs(fd), (name, fd, se, ad)


def test_c5_finite_differences_of_the_oracle_equal_the_renderer(c5):
    """The finite differences above are those of the reference's renderer: on a
    32 x 32 crop of the C5 film, the oracle's film at theta + eps v and at
    theta - eps v equals the GPU's bit for bit (albedo along a random direction,
    the alpha of the largest-gradient material, alpha along a random direction),
    so every finite difference of the oracle equals the renderer's."""
    from oracle.oracle import OracleScene
    d, s, st, prm, alb0, alpha0, w, set_params = c5
    crop = st.replace(spp=32, seed=100, x0=112, y0=112, width=32, height=32)
    _, g = d.adjoint_backward(st.replace(spp=256, seed=8), w, -1, prm["alpha_materials"])
    m = int(np.argmax(np.abs(g)))
    rng = np.random.default_rng(11)
    cases = [("albedo", alb0 + 1e-3 * rng.standard_normal(alb0.shape).astype(np.float32), alpha0),
             ("alpha", alb0, alpha0 * (1 + 0.05 * np.eye(alpha0.size)[m])),
             ("alpha", alb0, alpha0 * (1 - 0.05 * np.eye(alpha0.size)[m])),
             ("alpha", alb0, alpha0 * (1 + 0.02 * rng.standard_normal(alpha0.size)))]
    try:
        for name, alb, alpha in cases:
            set_params(alb.astype(np.float32), alpha)
            gpu = d.render(crop)
            orc = OracleScene(s)                  # the scene description carries the updated texels
            try:
                want = orc.render(crop)
            finally:
                orc.close()
            assert np.array_equal(gpu.view(np.uint32), want.view(np.uint32)), name
    finally:
        set_params(alb0, alpha0)
