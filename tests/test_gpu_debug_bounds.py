"""The debug-bounds build (gpu).

Built with -DRT_DEBUG_BOUNDS, the wavefront checks every computed index into its
path-state buffers (ray queues, active and sorted lists, per-sample radiance,
film splats): an index outside its buffer sets a status bit, the access is
skipped, and the call returns RT_ERR_BOUNDS.  This test builds that variant into
its own directory and runs the wavefront renderers over the parity scenes - with
the default slot pool and with a pool of 1000 slots, so slots are refilled many
times - in a child process that loads only that library.  Every call must
succeed and reproduce the oracle or the megakernel exactly as the default build
does.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import ctypes as C
import sys
import numpy as np
from radiantium_gb300 import native as N, procedural
from radiantium_gb300.device import Device
from oracle.oracle import OracleScene

lib = N.load_library()
assert lib._name == sys.argv[1], (lib._name, sys.argv[1])
MODES = [N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH]


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def limits(dev, capacity):
    f = dev.lib.rt_debug_set_limits
    f.restype, f.argtypes = C.c_int, [C.c_void_p, C.c_int64, C.c_int]
    assert f(dev.h, 0, capacity) == 0


def run(capacity):
    dev = Device(0)
    limits(dev, capacity)
    # path and vol_path against the oracle, both loop drivers
    for s, st in (procedural.cornell_box(48, 40), procedural.volume_box(32, 32),
                  procedural.material_zoo(32, 24)):
        st = st.replace(spp=4)
        dev.upload(s)
        want = OracleScene(s).render(st)
        for m in MODES:
            dev.set_renderer(m)
            assert np.array_equal(bits(dev.render(st)), bits(want)), (s.name, m)
    # a prototype deep enough for the shared-memory traversal stacks: wavefront == megakernel
    s, st = procedural.instanced_spheres(32, 24, sphere_n=64, grid=2, env_w=32, env_h=16)
    st = st.replace(spp=4)
    dev.upload(s)
    dev.set_renderer(N.RENDERER_MEGAKERNEL)
    want = dev.render(st)
    for m in MODES:
        dev.set_renderer(m)
        assert np.array_equal(bits(dev.render(st)), bits(want)), ("instanced", m)
    # the light tracer: films against the megakernel within the splat summation order
    s, st = procedural.cornell_box(40, 30)
    pst = st.replace(integrator=N.INTEGRATOR_PARTICLE)
    dev.upload(s)
    dev.set_renderer(N.RENDERER_MEGAKERNEL)
    want = dev.render_particles(pst, 40000).astype(np.float64)
    for m in MODES:
        dev.set_renderer(m)
        got = dev.render_particles(pst, 40000)
        assert np.allclose(got, want, rtol=1e-5, atol=1e-6 * want.max()), ("particles", m)
    # a batch of two scenes against their single renders
    a, sa = procedural.cornell_box(24, 20)
    b, sb = procedural.material_zoo(20, 16)
    da, db = Device(0), Device(0)
    da.upload(a)
    db.upload(b)
    sa, sb = sa.replace(spp=2), sb.replace(spp=2)
    films = dev.render_batch([(da, sa), (db, sb)])
    assert np.array_equal(bits(films[0]), bits(da.render(sa)))
    assert np.array_equal(bits(films[1]), bits(db.render(sb)))
    da.close()
    db.close()
    dev.close()


run(0)          # the default pool
run(1000)       # 1000 slots: every slot is refilled many times
print("debug-bounds ok")
'''


def test_debug_bounds_build(tmp_path):
    from radiantium_gb300 import build
    lib = build.build(extra_nvcc=["-DRT_DEBUG_BOUNDS"], out_dir=str(tmp_path / "debug_bounds"))
    env = dict(os.environ, RADIANTIUM_GB300_LIB=lib, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-c", CHILD, lib], env=env, cwd=ROOT, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "debug-bounds ok" in r.stdout
