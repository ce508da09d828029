"""The CUDA library against the committed golden fixtures (gpu).

The fixtures (tests/golden/, made by tests/golden/make_golden.py from the
oracle) are read as stored files: this module does not run the oracle.
Deterministic math, ray batches of a flat and an instanced scene, and film
crops of every method / strategy, the material zoo and a volume must match
bit for bit, with each renderer that runs the case.
"""
import os

import numpy as np
import pytest

from radiantium_gb300 import native as N
from tests.golden import make_golden

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DETMATH_FN = {"sin": 0, "cos": 1, "tan": 2, "atan": 3, "atan2": 4, "acos": 5, "exp": 6, "log": 7}


def _load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def test_detmath_golden(dev):
    g = _load("detmath")
    for name, fn in DETMATH_FN.items():
        out = dev.detmath(fn, g[name + "_a"], g[name + "_b"])
        assert np.array_equal(out.view(np.uint32), g[name + "_out"]), name


@pytest.mark.parametrize("case", make_golden.hit_cases(), ids=lambda c: c[0])
def test_hits_golden(dev, case):
    name, scene, _, _ = case
    g = _load("hits_" + name)
    dev.upload(scene)
    h = dev.trace_closest(g["rays"])
    for k in ("prim", "sub", "flags"):
        assert np.array_equal(h[k], g[k]), k
    for k in ("t", "u", "v"):
        assert np.array_equal(h[k].view(np.uint32), g[k]), k
    assert np.array_equal(dev.trace_any(g["rays"]).astype(np.uint8), g["occluded"])


@pytest.mark.parametrize("case", make_golden.film_cases(), ids=lambda c: c[0])
def test_films_golden(dev, case):
    name, scene, st = case
    want = _load("film_" + name)["film"]
    dev.upload(scene)
    modes = [N.RENDERER_MEGAKERNEL]
    if st.strategy == N.STRATEGY_UNIFORM or st.integrator == N.INTEGRATOR_PATH:
        modes += [N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH]
    try:
        for m in modes:
            dev.set_renderer(m)
            got = dev.render(st)
            assert np.array_equal(got.view(np.uint32), want), (name, m)
    finally:
        dev.set_renderer(N.RENDERER_AUTO)
