"""Generates the golden fixtures of tests/golden/ from the CPU oracle.

The reference (C#/.NET) cannot run in this image and ships no numeric
fixtures, so these vectors come from the oracle, the C++ restatement of the
reference's path.  They pin the oracle against regressions (CPU tests) and
let the GPU tests check the library against stored values without the
oracle.  Every input is seeded; re-running this script reproduces the files
bit for bit.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from radiantium_gb300 import native as N  # noqa: E402
from radiantium_gb300 import procedural  # noqa: E402
from oracle import oracle  # noqa: E402

DETMATH = {"sin": (-30, 30), "cos": (-30, 30), "tan": (-1.5, 1.5), "atan": (-50, 50), "atan2": (-3, 3),
           "acos": (-1, 1), "exp": (-90, 88), "log": (1e-30, 1e30)}


def rays_for(lo, hi, n, seed):
    """Rays from around the box towards points inside it (float32 ray records)."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    ext = hi - lo
    o = (lo + hi) / 2 + (rng.random((n, 3)) - 0.5) * ext * 3.0
    d = lo + rng.random((n, 3)) * ext - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(n, dtype=N.ray_dtype())
    rays["o"], rays["d"] = o.astype(np.float32), d.astype(np.float32)
    rays["min_t"] = np.float32(1e-4)
    rays["max_t"] = np.where(rng.random(n) < 0.8, 3.4028234663852886e38, rng.random(n) * 4).astype(np.float32)
    return rays


def hits_arrays(h):
    return {"prim": h["prim"], "sub": h["sub"], "t": h["t"].view(np.uint32), "u": h["u"].view(np.uint32),
            "v": h["v"].view(np.uint32), "flags": h["flags"]}


def film_cases():
    """(name, scene, settings) of the golden film crops."""
    cb, cst = procedural.cornell_box(256, 256)
    zoo, zst = procedural.material_zoo(48, 48)
    vol, vst = procedural.volume_box(40, 40)
    crop = dict(x0=100, y0=120, width=24, height=16, spp=32, seed=11)
    cases = []
    for name, m, strat in (("bxdf", N.METHOD_BXDF, N.STRATEGY_UNIFORM), ("nee", N.METHOD_NEE, N.STRATEGY_UNIFORM),
                           ("mis", N.METHOD_MIS, N.STRATEGY_UNIFORM), ("mis_all", N.METHOD_MIS, N.STRATEGY_ALL)):
        cases.append((f"cornell_{name}", cb, cst.replace(method=m, strategy=strat, **crop)))
    cases.append(("zoo_mis", zoo, zst.replace(x0=16, y0=16, width=16, height=16, spp=4, seed=5)))
    cases.append(("volume", vol, vst.replace(x0=12, y0=12, width=16, height=16, spp=4, seed=3)))
    return cases


def hit_cases():
    cb, _ = procedural.cornell_box(256, 256)
    inst, _ = procedural.instanced_spheres(96, 96, sphere_n=12, grid=4, env_w=64, env_h=32)
    return [("cornell", cb, ((0, 0, 0), (1, 1, 1)), 3),
            ("instanced", inst, ((-6, 0, -6), (6, 3, 6)), 4)]


def particle_cases():
    """(name, scene, settings) of the light-tracer fixtures: per-particle splats of
    particles [1000, 1512) and the film of particles [0, 20000) summed by one
    oracle thread (a fixed order)."""
    return [("cornell", *procedural.cornell_box(40, 30)),
            ("zoo", *procedural.material_zoo(32, 32)),
            ("instanced", *procedural.instanced_spheres(48, 32, sphere_n=12, grid=4, env_w=64, env_h=32))]


REFERENCE_SCENES = os.path.join(ROOT, "tests", "fixtures", "reference")


def reference_scene_cases():
    """(name, scene, settings) of the reference's own example scenes
    (tests/fixtures/reference): a 32 x 32 crop at the film's centre, 8 spp, for
    the path / vol_path scenes; the light-tracer scenes' settings for their
    per-particle splats."""
    from radiantium_gb300 import config
    from tests.fixtures.reference.copy_reference_scenes import SCENES
    cases = []
    for rel in SCENES:
        r = config.load_scene_file(os.path.join(REFERENCE_SCENES, rel))
        cam, st = r.scene.camera, r.settings
        name = rel.replace("/", "_").replace(".json", "")
        if st.integrator != N.INTEGRATOR_PARTICLE:
            st = st.replace(spp=8, seed=1, x0=cam.width // 2 - 16, y0=cam.height // 2 - 16, width=32, height=32)
        else:
            st = st.replace(seed=3)
        cases.append((name, r.scene, st))
    return cases


def generate():
    out = {}
    rng = np.random.default_rng(2024)
    # Philox streams (counter = pixel x, y, sample index; key = seed)
    ph = np.stack([oracle.philox_stream(s, x, y, t, 64) for s, x, y, t in
                   [(1, 0, 0, 0), (7, 13, 255, 3), (0xDEADBEEF, 1023, 1, 99), (2 ** 40 + 5, 7, 7, 7)]])
    out["philox"] = {"streams": ph.astype(np.uint32)}
    # deterministic math
    dm = {}
    for name, (lo, hi) in DETMATH.items():
        if name == "log":
            a = np.exp(rng.uniform(np.log(lo), np.log(hi), 1024)).astype(np.float32)
        else:
            a = rng.uniform(lo, hi, 1024).astype(np.float32)
        b = rng.uniform(-3, 3, 1024).astype(np.float32)
        dm[name + "_a"], dm[name + "_b"] = a, b
        dm[name + "_out"] = oracle.detmath(name, a, b).astype(np.float32).view(np.uint32)
    out["detmath"] = dm
    # ray batches
    for name, scene, (lo, hi), seed in hit_cases():
        orc = oracle.OracleScene(scene)
        rays = rays_for(lo, hi, 2048, seed)
        h = orc.trace_closest(rays)
        occ = orc.trace_any(rays)
        out[f"hits_{name}"] = dict(rays=rays, occluded=occ.astype(np.uint8), **hits_arrays(h))
        if name == "cornell":
            b = orc.bvh(-1)
            out["bvh_cornell"] = {k: np.asarray(v) for k, v in b.items()}
        orc.close()
    # film crops
    for name, scene, st in film_cases():
        orc = oracle.OracleScene(scene)
        film = orc.render(st)
        out[f"film_{name}"] = {"film": film.astype(np.float32).view(np.uint32)}
        orc.close()
    # light tracer (adjoint_particle)
    for name, scene, st in particle_cases():
        orc = oracle.OracleScene(scene)
        pst = st.replace(integrator=N.INTEGRATOR_PARTICLE, seed=5)
        n, pix, rgb = orc.particle_splats(pst, 512, 12, first=1000)
        film = orc.render_particles(pst, 20000, threads=1)
        out[f"particles_{name}"] = {"n": n, "pix": pix, "rgb": rgb.view(np.uint32),
                                    "film": film.astype(np.float32).view(np.uint32)}
        orc.close()
    # the reference's example scenes
    ref = {}
    for name, scene, st in reference_scene_cases():
        orc = oracle.OracleScene(scene)
        if st.integrator == N.INTEGRATOR_PARTICLE:
            n, pix, rgb = orc.particle_splats(st, 256, 12, first=77)
            ref[name + "_n"], ref[name + "_pix"], ref[name + "_rgb"] = n, pix, rgb.view(np.uint32)
        else:
            ref[name + "_film"] = orc.render(st).astype(np.float32).view(np.uint32)
        orc.close()
    out["reference_scenes"] = ref
    return out


def main():
    for name, arrays in generate().items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(name, {k: v.shape for k, v in arrays.items()})


if __name__ == "__main__":
    main()
