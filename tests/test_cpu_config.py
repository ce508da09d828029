"""The JSON scene loader (radiantium_gb300/config.py, the reference's
Config/RendererBuilder.cs registries and Radiantium.Cli/Program.cs GetRenderer)
on CPU: scene files in the reference's schema load into the flattened scene
with the reference's defaults, and the oracle renders what they describe.
The OBJ assets are small quads written by the test."""
import json

import numpy as np
import pytest

from radiantium_gb300 import native as N
from radiantium_gb300.config import load_scene_file, load_scene_file_with_output
from oracle import oracle as O


def _obj(path, quads):
    """Quads listed with outward normals, written reversed so that they face into the box."""
    lines, k = [], 1
    for q in quads:
        lines += [f"v {x} {y} {z}" for (x, y, z) in reversed(q)]
        lines += [f"f {k} {k + 1} {k + 2}", f"f {k} {k + 2} {k + 3}"]
        k += 4
    path.write_text("\n".join(lines) + "\n")


def _scene_file(tmp_path, integrator, renderer, extra_entities=(), instanced=None, medium=None):
    """A box open towards +z with a ceiling light, two spheres, in the reference's schema."""
    _obj(tmp_path / "walls.obj", [[(-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1)],     # floor
                                  [(-1, 1, -1), (-1, 1, 1), (1, 1, 1), (1, 1, -1)],         # ceiling
                                  [(-1, -1, -1), (-1, 1, -1), (1, 1, -1), (1, -1, -1)]])    # back
    _obj(tmp_path / "left.obj", [[(-1, -1, -1), (-1, -1, 1), (-1, 1, 1), (-1, 1, -1)]])
    _obj(tmp_path / "right.obj", [[(1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1)]])
    _obj(tmp_path / "light.obj", [[(-0.25, 0.99, -0.25), (-0.25, 0.99, 0.25), (0.25, 0.99, 0.25), (0.25, 0.99, -0.25)]])
    glob = {"outside": {"is_global": True}} if medium else None
    ents = [
        {"material": {"type": "diffuse", "kd": [0.7, 0.7, 0.7]}, "shape": {"type": "model", "name": "walls"}},
        {"material": {"type": "diffuse", "kd": [0.6, 0.1, 0.1]}, "shape": {"type": "model", "name": "left"}},
        {"material": {"type": "diffuse", "kd": [0.1, 0.6, 0.1]}, "shape": {"type": "model", "name": "right"}},
        {"material": {"type": "diffuse"}, "shape": {"type": "model", "name": "light"},
         "light": {"type": "diffuse_area", "le": [20, 20, 20]}},
        {"material": {"type": "perfect_glass"}, "shape": {"type": "sphere", "radius": 0.3, "center": [0.4, -0.7, 0.1]}},
        {"material": {"type": "perfect_mirror"}, "shape": {"type": "sphere", "radius": 0.3,
                                                          "center": [-0.4, -0.7, -0.3]}},
    ] + list(extra_entities)
    if glob:
        for e in ents:
            e["medium"] = dict(glob)
    cfg = {
        "renderer": renderer, "integrator": integrator,
        "camera": {"type": "perspective", "screen": [40, 30], "fov": 40, "far": 100,
                   "origin": [0, 0, 4.5], "target": [0, 0, 0], "up": [0, 1, 0]},
        "accel": {"type": "bvh"}, "output": {"save_name": "out"},
        "assets": [{"type": "model", "name": n, "location": f"{n}.obj"} for n in ("walls", "left", "right", "light")],
        "scene": ents,
    }
    if medium:
        cfg["camera"]["medium"] = medium
    if instanced is not None:
        cfg["instanced"] = instanced
    p = tmp_path / "scene.json"
    p.write_text(json.dumps(cfg))
    return str(p)


def test_path_scene_defaults_and_render(tmp_path):
    r, out = load_scene_file_with_output(_scene_file(tmp_path, {"type": "path", "max_depth": 5}, {"spp": 8}))
    s, st = r.scene, r.settings
    assert (s.camera.width, s.camera.height) == (40, 30)
    # RendererBuilder.cs:55-63 defaults: Mis, Uniform, min_depth 3, rr 0.99
    assert (st.integrator, st.method, st.strategy) == (N.INTEGRATOR_PATH, N.METHOD_MIS, N.STRATEGY_UNIFORM)
    assert (st.max_depth, st.min_depth, st.spp) == (5, 3, 8)
    assert abs(st.rr_threshold - 0.99) < 1e-7
    types = {m.type for m in s.materials}
    assert {N.MAT_DIFFUSE, N.MAT_PERFECT_GLASS, N.MAT_PERFECT_MIRROR} <= types
    assert sum(1 for g in s.groups if g.emissive) == 1
    assert out.save_name == "out"
    orc = O.OracleScene(s)
    try:
        img = orc.render(st.replace(spp=4))
    finally:
        orc.close()
    assert img.shape == (40, 30, 3) and np.isfinite(img).all() and img.mean() > 0.01


def test_particle_scene_selects_the_particle_renderer(tmp_path):
    """The integrator's TargetRendererName picks "adjoint_particle" (RendererBuilder.cs:523)."""
    r = load_scene_file(_scene_file(tmp_path, {"type": "adjoint_particle", "min_depth": 7},
                                    {"particle_count": 5000, "threads": -1}))
    st = r.settings
    assert st.integrator == N.INTEGRATOR_PARTICLE
    assert (st.max_depth, st.min_depth) == (-1, 7)
    assert r.particle_count == 5000 and r.AllTaskCount == 16
    orc = O.OracleScene(r.scene)
    try:
        img = orc.render_particles(st, 5000)
    finally:
        orc.close()
    assert np.isfinite(img).all() and img.mean() > 0.0


def test_gpu_renderer_mode_options(tmp_path):
    """The GPU renderer's own "renderer" keys: the opt-in wide traversal and
    alias-table env sampling; the reference's defaults when absent."""
    r = load_scene_file(_scene_file(tmp_path, {"type": "path"}, {"type": "gpu_wavefront", "spp": 4}))
    assert (r.traversal, r.light_sampling) == (N.TRAVERSAL_EXACT, N.LIGHT_SAMPLING_CDF)
    r = load_scene_file(_scene_file(tmp_path, {"type": "path"},
                                    {"type": "gpu_wavefront", "spp": 4, "traversal": "wide",
                                     "light_sampling": "alias"}))
    assert (r.traversal, r.light_sampling) == (N.TRAVERSAL_WIDE, N.LIGHT_SAMPLING_ALIAS)
    r = load_scene_file(_scene_file(tmp_path, {"type": "adjoint_particle"}, {"light_sampling": "alias"}))
    assert r.light_sampling == N.LIGHT_SAMPLING_ALIAS
    for bad in ({"traversal": "bvh4"}, {"light_sampling": "power"}):
        with pytest.raises(ValueError):
            load_scene_file(_scene_file(tmp_path, {"type": "path"}, dict(bad, spp=4)))


def test_particle_count_default(tmp_path):
    r = load_scene_file(_scene_file(tmp_path, {"type": "adjoint_particle"}, {}))
    assert r.particle_count == 16384      # RendererBuilder.cs:38


def test_vol_path_with_global_medium_and_instances(tmp_path):
    med = {"type": "homogeneous", "sigma_a": [0.01, 0.01, 0.01], "sigma_s": [0.05, 0.05, 0.05], "g": 0.3}
    inst = [{"shape": {"type": "model", "name": "left"}, "transform": {"scale": [0.3, 0.3, 0.3]}}]
    extra = [{"instanced": {"id": 0}, "transform": {"position": [0.5, 0.0, 0.3]}, "material": {"type": "diffuse"}}]
    r = load_scene_file(_scene_file(tmp_path, {"type": "vol_path", "max_depth": 6}, {"spp": 2}, extra, inst, med))
    s, st = r.scene, r.settings
    assert st.integrator == N.INTEGRATOR_VOL_PATH and st.max_depth == 6
    assert s.global_medium >= 0 and len(s.media) >= 1
    assert len(s.blas) == 1 and any(g.kind == N.GROUP_INSTANCE for g in s.groups)
    orc = O.OracleScene(s)
    try:
        img = orc.render(st.replace(x0=10, y0=10, width=8, height=8))
    finally:
        orc.close()
    assert np.isfinite(img).all()


@pytest.mark.parametrize("integrator", ["bdpt", "ao", "gbuffer"])
def test_plugins_outside_the_path_raise(tmp_path, integrator):
    with pytest.raises(NotImplementedError):
        load_scene_file(_scene_file(tmp_path, {"type": integrator}, {"spp": 4}))
