"""The opt-in fast traversal (RT_TRAVERSAL_WIDE) against the exact one (gpu).

The exact traversal is the reference's tree in the reference's order and is
shown equal to the oracle elsewhere; the fast one collapses the same trees
8-wide with quantised, outward-rounded child boxes.  Its contract, as the
tolerance for this path states it:

  * hit primitive ids equal the exact traversal's, with t, u, v bit for bit
    (the same Moller-Trumbore arithmetic on the same primitive), except where
    (a) two candidates are within 4 ulp of each other - exactly equal t
        (a tie), or coplanar surfaces a ulp apart of which the reference's
        box test culled the second at rounding scale - which the fast
        traversal meets and flags RT_HIT_TIE; the hit distance then stays
        within 4 ulp of the exact one, or
    (b) the fast traversal finds a hit more than 4 ulp closer: a primitive
        whose box the reference's slab test rejected at rounding scale (the
        fast boxes are conservative), or
    (c) the exact hit lies in an instance whose model-space MaxT is NaN for
        this unbounded ray: Ray3F.Transform (the reference's, restated by
        XfRay) maps MaxT = float.MaxValue through a world-to-model matrix
        with entries above 1 (an instance scaled below 1) to inf - inf, and
        the NaN MaxT culls the whole instance.  Whether the reference then
        sees the instance depends on whether a hit elsewhere made MaxT
        finite before the instance was entered - on traversal order - so
        the two traversals can differ there;
    exact ties are flagged; ties stay under 1 % of the rays (coplanar light
    and ceiling, boxes standing on the floor), (b) under 1 in 10,000, and
    every other disagreement is a case of (c);
  * any-hit answers are a superset of the exact ones (the same reason);
  * films differ from the exact films only in the paths that met such a ray:
    almost every float is identical and the relative mean squared difference
    is tiny.
Rays: 1 M per benchmark scene (camera rays and random rays through the
scene's box), 200 k for the small scenes.
"""
import numpy as np
import pytest

from radiantium_gb300 import native as N
from radiantium_gb300 import procedural
from oracle.oracle import OracleScene
from tests.test_gpu_parity import random_rays

pytestmark = pytest.mark.gpu

MAX_TIES = 1e-2         # rays whose hit is one of two candidates within 4 ulp
MAX_MISSES = 1e-4       # rays where the reference's slab test missed a closer hit
TIE_ULP = 4


def _scene(name):
    return {"cornell": lambda: procedural.cornell_box(256, 256),
            "zoo": lambda: procedural.material_zoo(64, 64),
            "C2": procedural.instanced_spheres,
            "C3": procedural.volume_sphere,
            "C4": lambda: procedural.batch_scene(8)}[name]()


def _rays(s, n, seed):
    orc = OracleScene(s)
    try:
        rng = np.random.default_rng(seed)
        cam = s.camera
        cam_rays = orc.camera_rays(rng.random((n // 2, 2)) * np.array([cam.width, cam.height]))
        root = orc.bvh(-1)["bounds"][0].astype(np.float64)
    finally:
        orc.close()
    box = (root[:3], root[3:])
    return np.concatenate([cam_rays, random_rays(box, n // 4, seed + 1),
                           random_rays(box, n - n // 2 - n // 4, seed + 2, inside=True)])


def _instance_of_prim(s):
    """Top-level primitive id -> the instance group it is, in build order."""
    out, pid = {}, 0
    for g in s.groups:
        if g.kind == N.GROUP_MESH:
            pid += s.meshes[g.ref].indices.shape[0]
        elif g.kind in (N.GROUP_SPHERE, N.GROUP_INSTANCE):
            if g.kind == N.GROUP_INSTANCE:
                out[pid] = g
            pid += 1
    return out


def _nan_model_maxt(ray, g):
    """XfRay's model-space MaxT of `ray` for instance group g is NaN (binary32,
    row-vector matrix, as the library computes it)."""
    f = np.float32
    m = np.asarray(g.model_to_world.invert().m, f).reshape(4, 4)
    with np.errstate(all="ignore"):
        o, d = ray["o"].astype(f), ray["d"].astype(f)
        p = o + f(ray["max_t"]) * d
        xf = lambda v: np.array([v[0] * m[0, c] + v[1] * m[1, c] + v[2] * m[2, c] + m[3, c] for c in range(3)], f)
        q = xf(p) - xf(o)
        return bool(np.isnan(np.sqrt(np.sum(q * q, dtype=f))))


def _trace(dev, rays, mode):
    dev.set_traversal(mode)
    try:
        assert dev.traversal() == mode
        return dev.trace_closest(rays), dev.trace_any(rays)
    finally:
        dev.set_traversal(N.TRAVERSAL_EXACT)


def _classify(name, s, rays, e, w, ea, wa):
    """Checks the contract above for one batch; returns (ties, slab misses, NaN culls)."""
    same = (e["prim"] == w["prim"]) & (e["sub"] == w["sub"])
    # the same primitive: the same arithmetic
    for k in ("t", "u", "v"):
        assert np.array_equal(e[k][same].view(np.uint32), w[k][same].view(np.uint32)), k
    diff = np.nonzero(~same)[0]
    inst = _instance_of_prim(s)
    ties = misses = nan_culls = 0
    for i in diff:
        et, wt = e["t"][i], w["t"][i]
        ulp = int(np.int64(np.float32(et).view(np.int32)) - np.int64(np.float32(wt).view(np.int32)))
        if e["prim"][i] >= 0 and w["prim"][i] >= 0 and abs(ulp) <= TIE_ULP:          # (a)
            ties += 1
            if ulp == 0:
                assert w["flags"][i] & N.HIT_TIE, ("an exact tie is flagged", i)
        elif w["prim"][i] >= 0 and (e["prim"][i] < 0 or wt < et):                    # (b)
            misses += 1
        else:                                                                         # (c)
            g = inst.get(int(e["prim"][i]))
            assert g is not None and _nan_model_maxt(rays[i], g), (name, i, rays[i], e[i], w[i])
            nan_culls += 1
    assert ties <= MAX_TIES * rays.size, (name, ties)
    assert misses <= MAX_MISSES * rays.size, (name, misses)
    # any hit: a superset of the exact answers
    assert not (ea.astype(bool) & ~wa.astype(bool)).any()
    assert int((wa.astype(bool) & ~ea.astype(bool)).sum()) <= MAX_MISSES * rays.size
    return ties, misses, nan_culls


@pytest.mark.parametrize("name", ["cornell", "zoo", "C2", "C3", "C4"])
def test_wide_hits_equal_exact_up_to_ties_and_slab_misses(dev, name):
    s, _ = _scene(name)
    dev.upload(s)
    n = 1 << 20 if name in ("C2", "C3") else 200000
    rays = _rays(s, n, 7)
    e, ea = _trace(dev, rays, N.TRAVERSAL_EXACT)
    w, wa = _trace(dev, rays, N.TRAVERSAL_WIDE)
    ties, misses, nan_culls = _classify(name, s, rays, e, w, ea, wa)
    print(f"{name}: {rays.size} rays, {ties} ties (within {TIE_ULP} ulp), {misses} reference slab misses, "
          f"{nan_culls} instances culled by a NaN model-space MaxT")
    assert (e["prim"] >= 0).sum() > rays.size // 10


def _axis_rays(s, n, seed):
    """Rays whose direction has exactly-zero components: a third along the six
    axes (two zeros, signed zeros included), the rest in the three coordinate
    planes (one zero), from points inside the scene's box."""
    orc = OracleScene(s)
    try:
        root = orc.bvh(-1)["bounds"][0].astype(np.float64)
    finally:
        orc.close()
    rng = np.random.default_rng(seed)
    lo, hi = root[:3], root[3:]
    o = lo + rng.random((n, 3)) * (hi - lo)
    d = np.zeros((n, 3))
    k = n // 3
    axis = rng.integers(0, 3, k)
    d[np.arange(k), axis] = rng.choice([-1.0, 1.0], k)
    a = rng.random(n - k) * 2 * np.pi
    zero = rng.integers(0, 3, n - k)
    for z in range(3):
        m = zero == z
        u, v = [c for c in range(3) if c != z]
        d[k:][m, u] = np.cos(a[m])
        d[k:][m, v] = np.sin(a[m])
    rays = np.zeros(n, dtype=N.ray_dtype())
    rays["o"] = o.astype(np.float32)
    dd = d.astype(np.float32)
    dd[dd == 0] = np.where(rng.random(int((dd == 0).sum())) < 0.5, 0.0, -0.0).astype(np.float32)
    rays["d"] = dd
    rays["min_t"] = 1e-4
    rays["max_t"] = np.float32(3.4028234663852886e38)
    return rays


@pytest.mark.parametrize("name", ["cornell", "C2", "C3"])
def test_wide_axis_parallel_rays(dev, name):
    """Directions with zero components (1/d infinite): the same contract, and
    the wide traversal visits fewer nodes than the exact one - a zero
    component must not make its boxes unbounded along that axis."""
    s, _ = _scene(name)
    dev.upload(s)
    rays = _axis_rays(s, 200000, 13)
    visits = {}
    res = {}
    dev.set_counting(True)
    try:
        for mode in (N.TRAVERSAL_EXACT, N.TRAVERSAL_WIDE):
            dev.set_traversal(mode)
            res[mode] = dev.trace_closest(rays)
            visits[mode] = dev.stats()["node_visits"]
            res[mode] = (res[mode], dev.trace_any(rays))
    finally:
        dev.set_counting(False)
        dev.set_traversal(N.TRAVERSAL_EXACT)
    (e, ea), (w, wa) = res[N.TRAVERSAL_EXACT], res[N.TRAVERSAL_WIDE]
    ties, misses, nan_culls = _classify(name, s, rays, e, w, ea, wa)
    print(f"{name}: {ties} ties, {misses} slab misses, {nan_culls} NaN culls; node visits per ray exact "
          f"{visits[N.TRAVERSAL_EXACT] / rays.size:.1f}, wide {visits[N.TRAVERSAL_WIDE] / rays.size:.1f}")
    assert (e["prim"] >= 0).sum() > rays.size // 10
    assert visits[N.TRAVERSAL_WIDE] < visits[N.TRAVERSAL_EXACT]


@pytest.mark.parametrize("name,spp", [("C2", 2), ("C3", 2), ("zoo", 16)])
def test_wide_films_match_exact(dev, name, spp):
    s, st = _scene(name)
    dev.upload(s)
    st = st.replace(spp=spp, sample_begin=3)
    if name == "C2":
        st = st.replace(x0=256, y0=256, width=512, height=512)
    films = []
    for mode in (N.TRAVERSAL_EXACT, N.TRAVERSAL_WIDE):
        dev.set_traversal(mode)
        try:
            films.append(dev.render(st))
        finally:
            dev.set_traversal(N.TRAVERSAL_EXACT)
    a, b = films
    assert np.isfinite(b).all()
    same = np.mean(a.view(np.uint32) == b.view(np.uint32))
    rel = float((((a.astype(np.float64) - b) ** 2) / (a.astype(np.float64) ** 2 + 1e-2)).mean())
    assert same >= 0.99, (name, same)
    assert rel <= 1e-4, (name, rel)


def test_wide_batch_equals_each_scene(dev):
    """A batch under the fast traversal reproduces each scene's own fast render."""
    from radiantium_gb300.device import Device
    scenes = [procedural.batch_scene(i) for i in (0, 3, 8)]
    devs = []
    try:
        for sc, _ in scenes:
            d = Device(0)
            d.upload(sc)
            d.set_traversal(N.TRAVERSAL_WIDE)
            devs.append(d)
        host = Device(0)
        host.set_traversal(N.TRAVERSAL_WIDE)
        items = [(d, st.replace(spp=1, sample_begin=2)) for d, (_, st) in zip(devs, scenes)]
        films = host.render_batch(items)
        for (d, st), f in zip(items, films):
            assert np.array_equal(f.view(np.uint32), d.render(st).view(np.uint32))
        host.close()
    finally:
        for d in devs:
            d.close()


def test_traversal_mode_arguments(dev):
    s, _ = _scene("cornell")
    dev.upload(s)
    with pytest.raises(N.RTError) as e:
        dev.set_traversal(7)
    assert e.value.code == N.RT_ERR_INVALID_ARG
    assert dev.traversal() == N.TRAVERSAL_EXACT
    dev.set_traversal(N.TRAVERSAL_WIDE)
    assert dev.traversal() == N.TRAVERSAL_WIDE
    dev.set_traversal(N.TRAVERSAL_EXACT)
