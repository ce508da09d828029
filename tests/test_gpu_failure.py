"""Failure paths of the renderers, made to happen on the host side or by
running a device loop out of its cap (gpu).  Nothing here faults or hangs a
GPU: every device loop has an iteration cap and reports it in the context's
status word, which the call turns into an error; the context stays usable.

  * the reference's 64-entry traversal stack (Accelerators/Bvh.cs:16,132,
    which throws on overflow): a scene whose SAH tree is 68 levels deep and a
    camera whose rays descend all of it -> RT_ERR_STACK from the megakernel
    and both wavefront loop drivers (and from the oracle);
  * Renderer.Stop (Renderers/BlockBasedRenderer.cs:84-88): rt_cancel from
    another host thread during a long render -> RT_ERR_CANCELLED, for each
    renderer;
  * the wavefront's bounce-iteration cap per round, lowered through a test
    hook -> RT_ERR_ITER_CAP from the host-driven and the graph-driven loop;
  * the per-path bounce cap, the traversal step cap and the null-boundary walk
    cap (caps the reference's loops do not have): a library built with tiny
    caps (RT_LOOP_CAP 16, RT_TRAVERSAL_CAP 48, RT_WALK_CAP 1) into its own
    directory, run in a child process that loads only it -> RT_ERR_ITER_CAP
    with the cap named, from every renderer that runs the loop.
After every failure the same context renders a scene that stays within the
caps and matches the oracle bit for bit.
"""
import ctypes as C
import os
import subprocess
import sys
import threading
import time

import numpy as np
import pytest

from radiantium_gb300 import native as N
from radiantium_gb300 import procedural
from radiantium_gb300.scene import Camera, Group, Material, Mesh, SceneDesc
from oracle.oracle import OracleScene

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MODES = (N.RENDERER_MEGAKERNEL, N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH)


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def deep_chain(width=16, height=16):
    """68 triangles whose SAH tree is one chain 68 levels deep: centroids at
    13^k on the x axis and at 13^(k - 33.5) on the y axis (k = 0..33), so every
    split peels off one triangle; each triangle's box spans x and z in +-1
    around it, so a ray along +y through the origin region hits the box of
    every remaining subtree and descends (pushing the peeled-off leaf) all the
    way down."""
    e = 1e-30
    s = SceneDesc(camera=Camera.look_at(width, height, 10.0, (0.0, -0.5, 0.0), (0.0, 1.0, 0.0), up=(0.0, 0.0, 1.0)),
                  name="deep_chain")
    pos = [(13.0 ** k, 0.0, 0.0) for k in range(34)] + [(0.0, 13.0 ** (k - 33.5), 0.0) for k in range(34)]
    p, idx = [], []
    for i, (x, y, z) in enumerate(pos):
        p += [(x - 1.0, y - e, z - 1.0), (x + 1.0, y - e, z + 1.0), (x, y + e, z)]
        idx.append((3 * i, 3 * i + 1, 3 * i + 2))
    mat = s.add_material(Material(N.MAT_DIFFUSE, tex_r=s.add_const(0.5)))
    s.groups.append(Group(N.GROUP_MESH, s.add_mesh(Mesh(np.asarray(p, np.float32), np.asarray(idx, np.int32))),
                          material=mat))
    env = s.add_const(1.0)
    s.groups.append(Group(N.GROUP_INFINITE_LIGHT, env))
    return s


def _usable(dev):
    """The context still renders: a Cornell crop equal to the oracle's."""
    s, st = procedural.cornell_box(32, 32)
    st = st.replace(spp=2)
    dev.upload(s)
    dev.set_renderer(N.RENDERER_AUTO)
    assert np.array_equal(_bits(dev.render(st)), _bits(OracleScene(s).render(st)))


def test_stack_overflow_on_a_68_level_tree(dev):
    s = deep_chain()
    st = procedural.cornell_box(16, 16)[1].replace(spp=1, max_depth=2)
    with pytest.raises(N.RTError) as e:
        OracleScene(s).render(st)
    assert e.value.code == N.RT_ERR_STACK, "the oracle (the reference's Bvh) overflows its stack"
    dev.upload(s)
    try:
        for m in MODES:
            dev.set_renderer(m)
            with pytest.raises(N.RTError) as e:
                dev.render(st)
            assert e.value.code == N.RT_ERR_STACK, m
            assert "stack" in str(e.value)
    finally:
        dev.set_renderer(N.RENDERER_AUTO)
    _usable(dev)


@pytest.mark.parametrize("mode", MODES)
def test_cancel_from_another_thread(dev, mode):
    s, st = procedural.instanced_spheres(512, 512, env_w=256, env_h=128)
    st = st.replace(spp=1024)                  # seconds of work on one GPU
    dev.upload(s)
    dev.set_renderer(mode)
    done = threading.Event()

    def stop():
        time.sleep(0.3)
        if not done.is_set():
            dev.cancel()

    t = threading.Thread(target=stop)
    t.start()
    try:
        t0 = time.perf_counter()
        with pytest.raises(N.RTError) as e:
            dev.render(st)
        done.set()
        assert e.value.code == N.RT_ERR_CANCELLED, mode
        assert time.perf_counter() - t0 < 20.0
    finally:
        done.set()
        t.join()
        dev.set_renderer(N.RENDERER_AUTO)
    _usable(dev)


def test_wavefront_iteration_cap(dev):
    s, st = procedural.cornell_box(32, 32)
    st = st.replace(spp=2, max_depth=8, min_depth=100)
    dev.upload(s)
    f = dev.lib.rt_debug_set_iter_cap
    f.argtypes, f.restype = [C.c_void_p, C.c_int], C.c_int
    try:
        assert f(dev.h, 3) == 0
        for m in (N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH):
            dev.set_renderer(m)
            with pytest.raises(N.RTError) as e:
                dev.render(st)
            assert e.value.code == N.RT_ERR_ITER_CAP, m
            assert "WF_ITER_CAP" in str(e.value)
    finally:
        assert f(dev.h, 0) == 0
        dev.set_renderer(N.RENDERER_AUTO)
    _usable(dev)


CHILD = r'''
import sys
import numpy as np
from radiantium_gb300 import native as N, procedural
from radiantium_gb300.device import Device
from radiantium_gb300.scene import Group, Mesh
from oracle.oracle import OracleScene

lib = N.load_library()
assert lib._name == sys.argv[1], (lib._name, sys.argv[1])
MODES = (N.RENDERER_MEGAKERNEL, N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH)
dev = Device(0)


def fails(s, st, cap, modes=MODES):
    dev.upload(s)
    for m in modes:
        dev.set_renderer(m)
        try:
            dev.render(st)
        except N.RTError as e:
            assert e.code == N.RT_ERR_ITER_CAP, (cap, m, e.code, str(e))
            assert cap in str(e), (cap, str(e))
        else:
            raise AssertionError(f"{cap}: renderer {m} did not report the cap")
    dev.set_renderer(N.RENDERER_AUTO)
    # the context still renders a scene that stays within the caps
    cb, cst = procedural.cornell_box(32, 32)
    cst = cst.replace(spp=2)
    dev.upload(cb)
    for m in MODES:
        dev.set_renderer(m)
        assert np.array_equal(dev.render(cst).view(np.uint32), OracleScene(cb).render(cst).view(np.uint32)), m
    dev.set_renderer(N.RENDERER_AUTO)


# bounce cap: unbounded depth, no Russian roulette before bounce 1000
cb, cst = procedural.cornell_box(32, 32)
fails(cb, cst.replace(spp=4, max_depth=-1, min_depth=1000), "RT_LOOP_CAP")
# traversal step cap: a leaf of 100 identical triangles in front of the camera
s, st = procedural.cornell_box(32, 32)
one = np.array([[0.3, 0.3, 0.5], [0.7, 0.3, 0.5], [0.5, 0.7, 0.5]], np.float32)
pile = Mesh(np.tile(one, (100, 1)), np.arange(300, dtype=np.int32).reshape(100, 3))
s.groups.append(Group(N.GROUP_MESH, s.add_mesh(pile), material=s.groups[0].material))
fails(s, st.replace(spp=1, max_depth=1), "RT_TRAVERSAL_CAP")
# null-boundary walk cap: vol_path walks through the medium's boundary
vs, vst = procedural.volume_box(24, 24)
fails(vs, vst.replace(spp=2, max_depth=4), "RT_WALK_CAP")
print("caps ok")
'''


def test_device_loop_caps(tmp_path):
    from radiantium_gb300 import build
    lib = build.build(extra_nvcc=["-DRT_LOOP_CAP=16", "-DRT_TRAVERSAL_CAP=48", "-DRT_WALK_CAP=1"],
                      out_dir=str(tmp_path / "small_caps"))
    env = dict(os.environ, RADIANTIUM_GB300_LIB=lib, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-c", CHILD, lib], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "caps ok" in r.stdout
