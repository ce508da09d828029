"""The reference's own example scenes through the scene loader and the oracle (CPU).

tests/fixtures/reference holds, byte for byte, the example scenes of
Radiantium (Example/**.json) whose assets the reference ships, with their OBJ
meshes (copy_reference_scenes.py; SHA-256 in MANIFEST.sha256).  Each one is
loaded through config.load_scene_file, the counterpart of the reference CLI's
GetRenderer (Radiantium.Cli/Program.cs:25-142) and RendererBuilder.Build, and
the flattened scene is checked against what the test reads from the JSON text
itself and against the reference's defaults:

  * integrator and renderer settings, with the defaults of
    Config/RendererBuilder.cs:29-40 (spp 256, particle_count 16384) and
    :56-79 (max_depth -1, min_depth 3, rr_threshold 0.99, method Mis,
    strategy Uniform);
  * the camera's screen, fov, near and far (RendererBuilder.cs:485-507:
    1280 x 720, 60, 0.001, 1000 by default);
  * one material per entity, of the JSON's type and parameters (the
    material builders of RendererBuilder.cs:80-200, including rough_metal's
    "metal_type" object, whose eta / k the reference reads from the material
    itself and so falls back to copper, RendererBuilder.cs:144-150);
  * the primitive list and Scene.Lights of the oracle: one primitive per
    sphere, per OBJ face and per instance in entity order, and one
    DiffuseAreaLight per primitive of an emissive entity with that entity's
    "le", as RendererBuilder.Build makes them (RendererBuilder.cs:943-993).
"""
import hashlib
import json
import os

import numpy as np
import pytest

from radiantium_gb300 import config
from radiantium_gb300 import native as N
from oracle.oracle import OracleScene
from tests.fixtures.reference.copy_reference_scenes import ASSETS, SCENES

FIXTURES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fixtures", "reference")
INTEGRATORS = {"path": N.INTEGRATOR_PATH, "vol_path": N.INTEGRATOR_VOL_PATH,
               "adjoint_particle": N.INTEGRATOR_PARTICLE}
METHODS = {"Mis": N.METHOD_MIS, "Nee": N.METHOD_NEE, "Bxdf": N.METHOD_BXDF}
MATERIALS = {"diffuse": N.MAT_DIFFUSE, "rough_metal": N.MAT_ROUGH_METAL, "rough_glass": N.MAT_ROUGH_GLASS,
             "rough_plastic": N.MAT_ROUGH_PLASTIC, "perfect_mirror": N.MAT_PERFECT_MIRROR,
             "perfect_glass": N.MAT_PERFECT_GLASS}
DISTS = {"GGX": N.DIST_GGX, "Beckmann": N.DIST_BECKMANN}
F32 = np.float32


def _json(rel):
    with open(os.path.join(FIXTURES, rel)) as f:
        return json.load(f)


def test_fixtures_are_the_reference_files():
    want = {}
    with open(os.path.join(FIXTURES, "MANIFEST.sha256")) as f:
        for line in f:
            digest, rel = line.split()
            want[rel] = digest
    assert set(want) == set(SCENES + ASSETS)
    for rel, digest in want.items():
        with open(os.path.join(FIXTURES, rel), "rb") as f:
            assert hashlib.sha256(f.read()).hexdigest() == digest, rel


def _obj_faces(rel_scene, location):
    path = os.path.normpath(os.path.join(FIXTURES, os.path.dirname(rel_scene), location))
    with open(path) as f:
        faces = [line.split()[1:] for line in f if line.startswith("f ")]
    assert all(len(v) == 3 for v in faces)
    return len(faces)


def _const(scene, tex):
    t = scene.textures[tex]
    assert (t.width, t.height) == (1, 1), "a constant texture"
    return t.data.reshape(3)


def _rgb(v):
    return np.asarray([v] * 3 if np.isscalar(v) else v, dtype=F32)


def _check_material(scene, mat, cfg):
    m = scene.materials[mat]
    t = cfg["type"]
    assert m.type == MATERIALS[t], t
    if t == "diffuse":
        assert np.array_equal(_const(scene, m.tex_r), _rgb(cfg.get("kd", 0.5)))
        assert m.two_sided == cfg.get("is_two_side", False)
    elif t in ("rough_metal", "rough_glass", "rough_plastic"):
        assert m.dist == DISTS[cfg.get("dist", "Beckmann" if t == "rough_plastic" else "GGX")]
        assert np.array_equal(_const(scene, m.tex_roughness), _rgb(cfg.get("roughness", 0.3)))
        assert np.array_equal(_const(scene, m.tex_anisotropic), _rgb(cfg.get("anisotropic", 0.0)))
        if t == "rough_metal":
            mt = cfg.get("metal_type", "Cu")
            eta, k = config.METALS[mt if isinstance(mt, str) else "Cu"]
            assert np.allclose(m.eta, eta, rtol=0, atol=0) and np.allclose(m.k, k, rtol=0, atol=0)
            assert m.two_sided == cfg.get("is_two_side", False)
        if t == "rough_plastic":
            assert np.array_equal(_const(scene, m.tex_r), _rgb(cfg.get("r", 0.5)))
            assert F32(m.kd) == F32(cfg.get("kd", 0.5)) and F32(m.ks) == F32(cfg.get("ks", 0.5))
        if t == "rough_glass":
            assert F32(m.eta_a) == F32(cfg.get("etaA", 1.000277)) and F32(m.eta_b) == F32(cfg.get("etaB", 1.5046))


def _expected_primitives_and_lights(rel, d):
    """Walks the JSON like RendererBuilder.Build: (primitive count, [(kind, prim, le)])."""
    models = {a["name"]: a["location"] for a in d.get("assets", []) if a["type"] == "model"}
    prims, lights = 0, []
    for e in d["scene"]:
        if "material" not in e and "medium" not in e:
            if "light" in e:
                lights.append((1, -1, (0.0, 0.0, 0.0)))
            continue
        n = 0
        shape = e.get("shape")
        if shape is not None:
            n = 1 if shape["type"] != "model" else _obj_faces(rel, models[shape["name"]])
        if "light" in e:
            le = tuple(float(F32(v)) for v in e["light"].get("le", (1.0, 1.0, 1.0)))
            lights.extend((0, prims + i, le) for i in range(n))
        prims += n + (1 if "instanced" in e else 0)
    return prims, lights


@pytest.mark.parametrize("rel", SCENES)
def test_reference_scene_flattens_like_the_reference(rel):
    d = _json(rel)
    r = config.load_scene_file(os.path.join(FIXTURES, rel))
    s, st = r.scene, r.settings
    ic, rc, cc = d["integrator"], d.get("renderer", {}), d["camera"]
    # integrator and renderer (RendererBuilder.cs:29-79)
    assert st.integrator == INTEGRATORS[ic["type"]]
    assert st.max_depth == ic.get("max_depth", -1)
    assert st.min_depth == ic.get("min_depth", 3)
    assert F32(st.rr_threshold) == F32(ic.get("rr_threshold", 0.99))
    if ic["type"] == "path":
        assert st.method == METHODS[ic.get("method", "Mis")]
    assert st.strategy == {"Uniform": N.STRATEGY_UNIFORM, "All": N.STRATEGY_ALL}[ic.get("strategy", "Uniform")]
    if ic["type"] == "adjoint_particle":
        assert r.particle_count == rc.get("particle_count", 16384)
    else:
        assert st.spp == rc.get("spp", 256)
    # camera (RendererBuilder.cs:485-507)
    cam = s.camera
    assert (cam.width, cam.height) == tuple(cc.get("screen", (1280, 720)))
    assert F32(cam.fov) == F32(cc.get("fov", 60.0))
    assert F32(cam.near) == F32(cc.get("near", 0.001)) and F32(cam.far) == F32(cc.get("far", 1000.0))
    # one material per entity that has one, in entity order, then instanced entities' materials
    mats = [g.material for g in s.groups if g.kind != N.GROUP_INFINITE_LIGHT]
    cfgs = [e["material"] for e in d["scene"] if "material" in e]
    used = []
    for m in mats:
        if m >= 0 and m not in used:
            used.append(m)
    assert len(used) == len(cfgs)
    for m, c in zip(used, cfgs):
        _check_material(s, m, c)
    # media: an entity with a medium gets an inside / outside medium as configured
    for e, g in zip([e for e in d["scene"] if "material" in e or "medium" in e],
                    [g for g in s.groups if g.kind != N.GROUP_INFINITE_LIGHT]):
        med = e.get("medium", {})
        inside, outside = med.get("inside", med.get("same")), med.get("outside", med.get("same"))
        for cfg, idx in ((inside, g.medium_inside), (outside, g.medium_outside)):
            if cfg is None:
                assert idx == -1
            elif cfg.get("is_global"):
                assert idx == s.global_medium
            else:
                mm = s.media[idx]
                assert np.array_equal(np.asarray(mm.sigma_a, F32), _rgb(cfg.get("sigma_a", 0.0)))
                assert np.array_equal(np.asarray(mm.sigma_s, F32), _rgb(cfg.get("sigma_s", 0.0)))
                assert F32(mm.g) == F32(cfg.get("g", 0.0)) and F32(mm.scale) == F32(cfg.get("scale", 1.0))
    # primitives and Scene.Lights, from the oracle's restated Build
    prims, lights = _expected_primitives_and_lights(rel, d)
    orc = OracleScene(s)
    try:
        assert orc.bvh(-1)["prim_order"].size == prims
        got = orc.lights()
        assert got["kind"].tolist() == [k for k, _, _ in lights]
        assert got["prim"].tolist() == [p for _, p, _ in lights]
        assert np.array_equal(got["le"], np.asarray([le for _, _, le in lights], F32).reshape(-1, 3))
        assert len(lights) > 0
    finally:
        orc.close()


def test_teapot_scene_is_instanced():
    """cbox/teapot.json renders two teapots through one instanced prototype (15,704 faces)."""
    d = _json("cbox/teapot.json")
    r = config.load_scene_file(os.path.join(FIXTURES, "cbox/teapot.json"))
    assert len(r.scene.blas) == len(d["instanced"]) == 1
    assert r.scene.meshes[r.scene.blas[0][0].ref].indices.shape[0] == _obj_faces("cbox/teapot.json",
                                                                                  "../assets/teapot.obj")
    inst = [g for g in r.scene.groups if g.kind == N.GROUP_INSTANCE]
    assert len(inst) == sum(1 for e in d["scene"] if "instanced" in e) >= 2
