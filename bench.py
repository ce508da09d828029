#!/usr/bin/env python3
"""Benchmark of the GB300 path tracer on the reference's headline workload.

Workload (default `instanced`): plain `path` integrator with MIS over 64
instances of a ~200k-triangle displaced sphere (GGX conductors with
alpha ~ U[0.05, 0.5] and rough dielectrics of IOR 1.5) lit by a 1024x512 HDR
environment of 8 Gaussian lobes; 1024x1024 pixels, 256 samples per pixel,
max depth 8.  The scene is generated from a seed (the reference ships none).

A step renders one progressive pass of `--spp-per-step` samples per pixel over
the whole film (the reference's BlockBasedRenderer sample loop, continued with
`sample_begin`), so the default 16 steps x 16 spp render exactly the 256-spp
frame.  `value` is device-resident throughput (samples/s) timed with CUDA
events; `e2e` renders the same passes through the C ABI call a host binding
makes (rt_render, film copied back to pinned host memory every step).

`--impl reference` times the reference's CPU path restated in C++ (oracle/,
all host cores) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import math
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "samples/s at fixed relMSE, batched vs plain GPU path; adjoint grads/s vs FD"
CLOCK_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                "clocks_event_reasons.sw_power_cap")
# algorithmic bytes (reference layout): ray record in + hit out per traced ray,
# one 32-byte LinearBVHNode per box test, 48 bytes per primitive test
# (3 indices + 3 positions), two 4x4 matrices per instance traversal,
# one 12-byte film write per sample.
B_RAY, B_NODE, B_PRIM, B_INST, B_FILM = 48, 32, 48, 128, 12


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=16)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["instanced", "cornell", "volume", "batch", "adjoint", "particle"],
                    default="instanced")
    ap.add_argument("--particles-per-step", type=int, default=1 << 24, help="particle workload: particles per step")
    ap.add_argument("--spp-per-step", type=int, default=16)
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="target length of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--renderer", choices=["auto", "megakernel", "wavefront", "graph"], default="auto")
    ap.add_argument("--traversal", choices=["exact", "wide"], default="exact",
                    help="exact: the reference's tree and order (bit-exact films); wide: the opt-in fast traversal")
    ap.add_argument("--light-sampling", choices=["cdf", "alias"], default="cdf",
                    help="cdf: the reference's CDF search (bit-exact films); alias: opt-in alias tables (same pmf)")
    ap.add_argument("--no-fd-check", action="store_true", help="adjoint workload: skip the finite-difference check")
    ap.add_argument("--no-relmse", action="store_true", help="skip the converged render for relMSE")
    ap.add_argument("--no-subrecords", action="store_true",
                    help="instanced workload: skip the batch and adjoint sub-records after the headline timing")
    ap.add_argument("--autotune", choices=["on", "off"], default="off",
                    help="path workloads: pick the wavefront settings with rt_autotune on one step (untimed); "
                         "off by default: the defaults were as fast on C1-C3, and a 1-spp probe picked settings "
                         "that lose on full steps")
    ap.add_argument("--plain-steps", type=int, default=2,
                    help="steps of the plain megakernel timed in the same run for the batched/plain ratio (0: skip)")
    return ap.parse_args()


def workload(name):
    from radiantium_gb300 import procedural
    if name == "adjoint":
        scene, st, _ = procedural.adjoint_patches()
        return scene, st
    scene, st = {"instanced": procedural.instanced_spheres, "cornell": procedural.cornell_box,
                 "volume": procedural.volume_sphere}[name]()
    return scene, st


def workload_config(name, scene, st, spp_step):
    from radiantium_gb300 import native as N
    return {
        "workload": {"instanced": "path MIS, 64 instances of a displaced sphere (GGX conductor / rough dielectric), "
                                  "1024x512 Gaussian-lobe env",
                     "adjoint": "forward renders of the adjoint workload's scene (64 rough_plastic patches, 512x512 "
                                "albedo texture): the reference has no derivatives, finite differences need two "
                                "renders per parameter",
                     "cornell": "path MIS, procedural Cornell box (36 tris, ceiling quad light)",
                     "volume": "vol_path, displaced sphere (499,392 triangles) bounding a homogeneous medium, ground, "
                               "quad light"}[name],
        "film": [scene.camera.width, scene.camera.height],
        "spp_frame": st.spp,
        "spp_per_step": spp_step,
        "max_depth": st.max_depth,
        "integrator": "vol_path" if st.integrator == N.INTEGRATOR_VOL_PATH else "path",
        "triangles": scene.triangle_count,
        "seed": st.seed,
    }


CPU_GRID, CPU_TILE = 8, 8      # the CPU samples: an 8 x 8 grid of 8 x 8 tiles spread over the film


def cpu_tiles(scene):
    """Origins of the CPU sample's tiles: the centres of an 8 x 8 grid over the
    film, so that background, edges and the dense middle are all in the sample
    (the reference renders a pixel's samples one after another, and so does
    each tile)."""
    W, H = scene.camera.width, scene.camera.height
    size = min(CPU_TILE, W, H)
    tiles = []
    for i in range(CPU_GRID):
        for j in range(CPU_GRID):
            x0 = min(W - size, max(0, int(round((i + 0.5) * W / CPU_GRID - size / 2))))
            y0 = min(H - size, max(0, int(round((j + 0.5) * H / CPU_GRID - size / 2))))
            tiles.append((x0, y0))
    return size, tiles


def oracle_tiles(orc, st, size, tiles, spp, begin, cores):
    """Renders every tile at `spp` samples per pixel from sample index `begin`
    on `cores` host threads; returns the samples rendered.  The work is cut into
    (tile, sample range) items of one oracle thread each, taken dynamically, so
    cheap and expensive tiles keep every core busy."""
    from concurrent.futures import ThreadPoolExecutor
    chunk = max(1, spp // 4)
    items = [(x0, y0, b, min(chunk, spp - b)) for (x0, y0) in tiles for b in range(0, spp, chunk)]

    def one(it):
        x0, y0, b, n = it
        orc.render(st.replace(spp=n, sample_begin=begin + b, x0=x0, y0=y0, width=size, height=size), threads=1)

    with ThreadPoolExecutor(max_workers=cores) as ex:
        list(ex.map(one, items))
    return len(tiles) * size * size * spp


def tiles_work(orc, st, size, tiles, cores):
    """Node visits per sample of the tiles at 1 spp (untimed): how the sample's
    traversal work compares with the whole film's."""
    from concurrent.futures import ThreadPoolExecutor

    def one(t):
        _, c = orc.render(st.replace(spp=1, x0=t[0], y0=t[1], width=size, height=size), threads=1, stats=True)
        return c["node_visits"], c["samples"]

    with ThreadPoolExecutor(max_workers=cores) as ex:
        r = list(ex.map(one, tiles))
    return sum(a for a, _ in r) / max(1, sum(b for _, b in r))


def tiles_desc(size, tiles, spp):
    return (f"{len(tiles)} tiles of {size}x{size} pixels on a {CPU_GRID}x{CPU_GRID} grid over the film x {spp} spp "
            f"({len(tiles) * size * size * spp} samples)")


def cpu_baseline(scene, st, target_s, threads=0, frame_nodes_per_sample=None):
    """Times the CPU oracle (the reference path restated in C++) on a bounded
    sample of the same workload: 64 tiles spread over the film, all host cores.
    frame_nodes_per_sample: the whole film's traversal work per sample (from the
    GPU's counting pass), reported beside the sample's own."""
    from oracle.oracle import OracleScene
    cores = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    orc = OracleScene(scene)
    build_s = time.perf_counter() - t0
    size, tiles = cpu_tiles(scene)
    t0 = time.perf_counter()
    oracle_tiles(orc, st, size, tiles, 1, 0, cores)
    t1 = time.perf_counter() - t0
    spp = int(max(1, min(st.spp, target_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    samples = oracle_tiles(orc, st, size, tiles, spp, 1, cores)
    dt = time.perf_counter() - t0
    work = tiles_work(orc, st, size, tiles, cores)
    orc.close()
    return {"value": samples / dt, "unit": "samples/s", "cores": cores, "kind": "port",
            "sample": f"{tiles_desc(size, tiles, spp)} of the same workload ({dt:.1f} s; oracle scene build "
                      f"{build_s:.1f} s not timed)",
            "sample_nodes_per_sample": work, "frame_nodes_per_sample": frame_nodes_per_sample}


class ClockSampler:
    """nvidia-smi sampling during the timed region (every 200 ms)."""

    def __init__(self, gpu_index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={CLOCK_FIELDS}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, reasons, mx = [], set(), None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "fallback 6.8 TB/s"


def profiled_traffic(name, key="bytes_per_sample"):
    """A figure of the traversal kernels from the committed ncu summary
    (profiles/trace_<workload>_traffic.txt: one line `<key>=<x>`): per-sample (or
    per-particle) DRAM traffic by default, or the limiter figures of the
    one-kernel capture."""
    p = os.path.join(ROOT, "profiles", f"trace_{name}_traffic.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(key + "="):
            return float(line.split("=", 1)[1])
    return None


def cpu_baseline_batch(scenes, step_settings, target_s, threads=0):
    """The CPU oracle over every scene of the batch: each scene timed on its own
    spread-tile sample (about target_s / n seconds each, all host cores), and
    the rates combined with one batch step's sample counts - the CPU time of a
    step is the sum over scenes of (the scene's samples in the step / its rate)."""
    from oracle.oracle import OracleScene
    cores = threads or os.cpu_count() or 1
    # at least half a second per scene: a tile call's fixed cost must not count
    per = max(target_s / len(scenes), 0.5)
    step_samples, cpu_s, sampled, timed_s, build_s = 0, 0.0, 0, 0.0, 0.0
    for (scene, _), st in zip(scenes, step_settings):
        t0 = time.perf_counter()
        orc = OracleScene(scene)
        build_s += time.perf_counter() - t0
        size, tiles = cpu_tiles(scene)
        t0 = time.perf_counter()
        oracle_tiles(orc, st, size, tiles, 16, 0, cores)
        t16 = time.perf_counter() - t0
        # samples beyond the step's own spp (the next sample indices of the same
        # pixels), so that every scene's sample is long enough to time
        spp = int(max(16, min(4096, 16 * per / max(t16, 1e-3))))
        t0 = time.perf_counter()
        n = oracle_tiles(orc, st, size, tiles, spp, 16, cores)
        dt = time.perf_counter() - t0
        orc.close()
        s_step = scene.camera.width * scene.camera.height * st.spp
        step_samples += s_step
        cpu_s += s_step * dt / n
        sampled += n
        timed_s += dt
    return {"value": step_samples / cpu_s, "unit": "samples/s", "cores": cores, "kind": "port",
            "sample": (f"every scene of the batch: {CPU_GRID * CPU_GRID} tiles of up to {CPU_TILE}x{CPU_TILE} "
                       f"pixels spread over each film, {sampled} samples in all ({timed_s:.1f} s; oracle scene "
                       f"builds {build_s:.1f} s not timed); the scenes' rates weighted by a batch step's samples")}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    scene, st = workload(args.workload)
    from oracle.oracle import OracleScene
    cores = os.cpu_count() or 1
    orc = OracleScene(scene)
    size, tiles = cpu_tiles(scene)
    t0 = time.perf_counter()
    oracle_tiles(orc, st, size, tiles, 1, 0, cores)
    t1 = time.perf_counter() - t0
    # each step: a bounded sample sized so the whole run stays within a few minutes
    total_steps = args.steps + args.warmup
    spp = int(max(1, min(st.spp, (150.0 / total_steps) / max(t1, 1e-3))))
    for i in range(args.warmup):
        oracle_tiles(orc, st, size, tiles, spp, i * spp, cores)
    times = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        samples = oracle_tiles(orc, st, size, tiles, spp, (args.warmup + i) * spp, cores)
        times.append(time.perf_counter() - t0)
    work = tiles_work(orc, st, size, tiles, cores)
    orc.close()
    ms = 1000.0 * float(np.mean(times))
    value = samples / (ms / 1000.0)
    sample_desc = tiles_desc(size, tiles, spp) + " per step"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": workload_config(args.workload, scene, st, args.spp_per_step),
        "run": {"step": sample_desc, "parallelism": f"{cores} host threads"},
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": cores, "kind": "port",
                         "sample": sample_desc + "; the C# reference cannot run here (no .NET), its C++ restatement "
                                                 "(oracle/) runs on all host cores",
                         "sample_nodes_per_sample": work},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    from radiantium_gb300.device import Device

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    from radiantium_gb300 import native as N
    scene, st = workload(args.workload)
    t0 = time.perf_counter()
    dev = Device(local)
    dev.upload(scene)
    mode = {"auto": N.RENDERER_AUTO, "megakernel": N.RENDERER_MEGAKERNEL, "wavefront": N.RENDERER_WAVEFRONT,
            "graph": N.RENDERER_WAVEFRONT_GRAPH}[args.renderer]
    dev.set_renderer(mode)
    traversal = N.TRAVERSAL_WIDE if args.traversal == "wide" else N.TRAVERSAL_EXACT
    light_sampling = N.LIGHT_SAMPLING_ALIAS if args.light_sampling == "alias" else N.LIGHT_SAMPLING_CDF
    uses_wavefront = mode in (N.RENDERER_WAVEFRONT, N.RENDERER_WAVEFRONT_GRAPH) or (
        mode == N.RENDERER_AUTO and st.strategy == N.STRATEGY_UNIFORM)
    upload_s = time.perf_counter() - t0
    W, H = scene.camera.width, scene.camera.height
    npix = W * H
    spp_step = args.spp_per_step
    # each rank renders its own sample passes (independent, no exchange): weak scaling
    base = rank * (args.warmup + args.steps) * spp_step
    film = torch.empty(npix * 3, dtype=torch.float32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream

    # untimed, optional: the film-preserving wavefront settings (slots in flight, trace-warp
    # refill, host- or graph-driven loop) picked by rt_autotune on one step of this workload
    tuned = None
    if uses_wavefront and mode == N.RENDERER_AUTO and args.autotune == "on":
        tuned = dev.autotune([(dev, st.replace(spp=spp_step, sample_begin=base))])
    # the library's AUTO rule: vol_path (and an autotune that picked it) runs the graph-driven loop
    graph_loop = mode == N.RENDERER_WAVEFRONT_GRAPH or (mode == N.RENDERER_AUTO and (
        st.integrator == N.INTEGRATOR_VOL_PATH or (tuned is not None and tuned["renderer"] == N.RENDERER_WAVEFRONT_GRAPH)))

    # one untimed counting pass: exact traversal counts of this workload
    dev.set_counting(True)
    dev.render_device(st.replace(spp=spp_step, sample_begin=base), film.data_ptr(), stream)
    torch.cuda.synchronize()
    counts = dev.stats()
    dev.set_counting(False)

    dev.set_traversal(traversal)            # the counting pass above ran the exact traversal
    dev.set_light_sampling(light_sampling)
    for i in range(args.warmup):
        dev.render_device(st.replace(spp=spp_step, sample_begin=base + i * spp_step), film.data_ptr(), stream)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    step_ms, kernel_ms, shade_ms, launches, render_launches = [], 0.0, 0.0, 0, 0
    frame = torch.zeros_like(film)
    for i in range(args.steps):
        flush.fill_(float(i))  # L2 flush between timed steps, outside the events
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        dev.render_device(st.replace(spp=spp_step, sample_begin=base + (args.warmup + i) * spp_step),
                          film.data_ptr(), stream)
        e1.record()
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        frame += film                          # the steps' passes average to the frame (outside the events)
        s = dev.stats()
        kernel_ms += s["render_kernel_ms"]
        shade_ms += s["shade_kernel_ms"]
        launches += s["kernel_launches"]
        render_launches += s["render_launches"]
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    total_ms = float(np.sum(step_ms))
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / args.steps
    samples_step = npix * spp_step
    value = samples_step * world / (ms_step / 1000.0)

    # relMSE of the frame the timed steps rendered, against an independent render
    # at 8x its spp (a converged-reference comparison; films of every renderer
    # here are identical per sample, so equal spp means equal relMSE)
    relmse = None
    if not args.no_relmse:
        frame_spp = spp_step * args.steps
        ref = torch.empty_like(film)
        dev.render_device(st.replace(spp=8 * frame_spp, sample_begin=0, seed=st.seed + 7919), ref.data_ptr(), stream)
        torch.cuda.synchronize()
        x, r = (frame / args.steps).double(), ref.double()
        relmse = {"value": float((((x - r) ** 2) / (r ** 2 + 1e-2)).mean().item()), "frame_spp": frame_spp,
                  "reference_spp": 8 * frame_spp,
                  "definition": "mean over pixels and channels of (x - r)^2 / (r^2 + 0.01); r independent seeds"}

    # e2e: the C ABI call a host binding makes, film copied to pinned host memory each step
    e2e = None
    if not args.no_e2e:
        host = torch.empty(npix * 3, dtype=torch.float32, pin_memory=True).numpy()
        import ctypes as C
        p = host.ctypes.data_as(C.c_void_p)
        lib, h = dev.lib, dev.h
        times, h2d = [], []
        for i in range(args.steps):
            prm = st.replace(spp=spp_step, sample_begin=base + (args.warmup + args.steps + i) * spp_step).to_c()
            t0 = time.perf_counter()
            rc = lib.rt_render(h, C.byref(prm), p)
            times.append(time.perf_counter() - t0)
            if rc != 0:
                raise RuntimeError(lib.rt_last_error(h).decode())
            h2d.append(dev.stats()["h2d_bytes"])     # job tables and queue counters the call copied
        e2e_s = float(np.mean(times))
        e2e = {"value": samples_step * world / e2e_s, "unit": "samples/s", "h2d_bytes_per_step": int(np.mean(h2d)),
               "d2h_bytes_per_step": npix * 12,
               "note": "rt_render with a pinned host film; scene resident (rt_upload_scene once, "
                       f"{upload_s:.2f} s incl. BVH builds); h2d = the job tables and queue counters the "
                       "call copies (rt_stats.h2d_bytes)"}

    # the opt-in wide traversal on the same passes (the headline stays on the exact one)
    wide = alias = both = None
    if uses_wavefront and traversal == N.TRAVERSAL_EXACT and light_sampling == N.LIGHT_SAMPLING_CDF \
            and not args.no_subrecords and rank == 0:
        sub = lambda t, l: mode_subrecord(dev, st, spp_step, base + args.warmup * spp_step, film, flush, stream,
                                          value, ms_step, t, l)
        wide = sub(N.TRAVERSAL_WIDE, N.LIGHT_SAMPLING_CDF)
        if any(g.kind == N.GROUP_INFINITE_LIGHT for g in scene.groups):
            alias = sub(N.TRAVERSAL_EXACT, N.LIGHT_SAMPLING_ALIAS)
            both = sub(N.TRAVERSAL_WIDE, N.LIGHT_SAMPLING_ALIAS)

    # the plain megakernel on the same passes, for the wavefront / megakernel ratio
    plain = None
    if uses_wavefront and args.plain_steps > 0:
        dev.set_renderer(N.RENDERER_MEGAKERNEL)
        pt = []
        for i in range(args.plain_steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dev.render_device(st.replace(spp=spp_step, sample_begin=base + (args.warmup + i) * spp_step),
                              film.data_ptr(), stream)
            e1.record()
            e1.synchronize()
            pt.append(e0.elapsed_time(e1))
        dev.set_renderer(mode)
        plain = {"value": samples_step / (float(np.mean(pt)) / 1000.0), "unit": "samples/s", "steps": args.plain_steps,
                 "note": "plain megakernel (one thread per camera sample), same passes, identical films"}

    # roofline of the path-tracing kernel (algorithmic bytes from exact counts); a
    # graph-driven loop is timed as a whole, so the trace kernels' own time then
    # comes from one more (untimed) step of the host-driven loop
    alg_bytes_step = (B_RAY * (counts["rays_closest"] + counts["rays_shadow"]) + B_NODE * counts["node_visits"]
                      + B_PRIM * counts["prim_tests"] + B_INST * counts["instance_visits"] + B_FILM * counts["samples"])
    if graph_loop:
        dev.set_renderer(N.RENDERER_WAVEFRONT)
        dev.render_device(st.replace(spp=spp_step, sample_begin=base + args.warmup * spp_step), film.data_ptr(), stream)
        torch.cuda.synchronize()
        s = dev.stats()
        kernel_ms, shade_ms = s["render_kernel_ms"] * args.steps, s["shade_kernel_ms"] * args.steps
        render_launches = s["render_launches"] * args.steps
        dev.set_renderer(mode)
    # wavefront: every traversal launch of a step together traces the step's rays,
    # so the roofline uses the step's algorithmic bytes over its summed traversal time
    launches_per_step = max(1, render_launches // args.steps)
    launch_ms = kernel_ms / max(1, render_launches)
    achieved = alg_bytes_step / (kernel_ms / args.steps / 1000.0) / 1e9
    peak, peak_src = measured_peak()
    tps = profiled_traffic(args.workload) if uses_wavefront else None
    # the limiter of the trace kernels, from the committed one-kernel capture
    l2f = profiled_traffic(args.workload, "l2_throughput_frac") if uses_wavefront else None
    lanes = profiled_traffic(args.workload, "threads_per_warp_instruction") if uses_wavefront else None
    issue = profiled_traffic(args.workload, "issue_slots_busy_frac") if uses_wavefront else None
    traffic = None if tps is None else tps * samples_step / launches_per_step
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(scene, st, args.cpu_seconds,
                           frame_nodes_per_sample=counts["node_visits"] / max(1, counts["samples"]))
    if relmse is not None:
        # time to reach this relMSE: every arm computes the same per-sample values,
        # so each needs the frame's samples, at its own rate
        frame_samples = samples_step * args.steps
        relmse["seconds_to_reach"] = {
            "gpu": args.steps * ms_step / 1000.0,
            "gpu_e2e": frame_samples * world / e2e["value"] if e2e else None,
            "plain_megakernel": frame_samples / plain["value"] if plain else None,
            "cpu": frame_samples / cpu["value"] if cpu else None}

    line = {
        "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": workload_config(args.workload, scene, st, spp_step),
        "run": {"parallelism": f"replicas x{world} (independent sample passes)",
                "l2": "256 MiB flush between timed steps (outside the CUDA events)",
                "renderer": ("wavefront (trace / shade kernels over compacted queues, path regeneration)"
                             + (", bounce loop as a CUDA graph" if graph_loop else "")
                             if uses_wavefront else "plain megakernel (one thread per camera sample)"),
                "autotune": tuned,
                "traversal": ("exact (the reference's tree and visit order)" if traversal == N.TRAVERSAL_EXACT
                              else "wide (opt-in fast traversal; the counting pass and algorithmic bytes use "
                                   "the exact one)"),
                "light_sampling": ("cdf (the reference's CDF search)" if light_sampling == N.LIGHT_SAMPLING_CDF
                                   else "alias (opt-in alias tables, the same texel pmf; the counting pass uses "
                                        "the CDF search)")},
        "mrays_per_s": (counts["rays_closest"] + counts["rays_shadow"]) * world / (ms_step / 1000.0) / 1e6,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_src,
                     "kernel": "k_wf_trace_closest + k_wf_trace_shadow" if uses_wavefront else "k_render",
                     "alg_bytes_per_launch": alg_bytes_step / launches_per_step, "launch_ms": launch_ms,
                     "launches_per_step": launches_per_step,
                     "kernel_ms_per_step": kernel_ms / args.steps, "shade_ms_per_step": shade_ms / args.steps,
                     "l2_frac": l2f, "lanes_per_instr": lanes, "issue_slots_busy": issue,
                     "limiter_source": (f"profiles/trace_{args.workload}_traffic.txt (ncu --set full, one launch of "
                                        "k_wf_trace_closest)") if l2f is not None else None},
        "plain_megakernel": plain,
        "wide_traversal": wide,
        "alias_light_sampling": alias,
        "wide_traversal_and_alias_light_sampling": both,
        "relmse": relmse,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
        "counts_per_step": {k: counts[k] for k in ("samples", "rays_closest", "rays_shadow", "node_visits",
                                                   "prim_tests", "instance_visits", "invalid_samples")},
    }
    dev.close()
    del film, flush, frame
    if args.workload == "instanced" and world == 1 and not args.no_subrecords:
        line["batch"] = batch_subrecord(args, rank, world, local, dist)
        line["adjoint"] = adjoint_subrecord(args, rank, world, local, dist)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def mode_subrecord(dev, st, spp_step, begin, film, flush, stream, exact_value, exact_ms, traversal, light_sampling,
                   steps=4, warmup=2):
    """The same passes with opt-in modes: the wide traversal (RT_TRAVERSAL_WIDE)
    and / or alias-table environment sampling (RT_LIGHT_SAMPLING_ALIAS).  Their
    samples/s against the default modes'; for the wide traversal alone, how far
    one pass's film is from the exact film (share of identical floats, relative
    mean squared difference) - alias sampling maps uniforms to other texels, so
    its films agree only statistically (tests/test_gpu_alias.py)."""
    import torch
    from radiantium_gb300 import native as N
    wide = traversal == N.TRAVERSAL_WIDE
    dev.set_traversal(traversal)
    if dev.traversal() != traversal:
        dev.set_traversal(N.TRAVERSAL_EXACT)
        return {"available": False, "note": "the scene's wide trees could overflow the traversal stack"}
    dev.set_light_sampling(light_sampling)
    try:
        for i in range(warmup):
            dev.render_device(st.replace(spp=spp_step, sample_begin=begin + i * spp_step), film.data_ptr(), stream)
        torch.cuda.synchronize()
        times, trace = [], 0.0
        for i in range(steps):
            flush.fill_(float(i))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dev.render_device(st.replace(spp=spp_step, sample_begin=begin + i * spp_step), film.data_ptr(), stream)
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
            trace += dev.stats()["render_kernel_ms"]
        ms = float(np.mean(times))
        mode_film = film.clone()
    finally:
        dev.set_traversal(N.TRAVERSAL_EXACT)
        dev.set_light_sampling(N.LIGHT_SAMPLING_CDF)
    value = exact_value * exact_ms / ms
    out = {"available": True, "value": value, "unit": "samples/s", "steps": steps, "ms_per_step": ms,
           "trace_ms_per_step": trace / steps, "vs_default": value / exact_value}
    notes = []
    if wide:
        notes.append("rt_set_traversal(RT_TRAVERSAL_WIDE): the same trees collapsed 8-wide with quantised child "
                     "boxes; hits equal the exact traversal's up to ties within 4 ulp and rounding-scale box culls "
                     "of the reference (tests/test_gpu_wide_traversal.py)")
    if light_sampling == N.LIGHT_SAMPLING_ALIAS:
        notes.append("rt_set_light_sampling(RT_LIGHT_SAMPLING_ALIAS): O(1) alias picks with exactly the CDF "
                     "search's texel pmf over the 2^24 uniforms (tests/test_cpu_alias.py, tests/test_gpu_alias.py)")
    if wide and light_sampling == N.LIGHT_SAMPLING_CDF:
        dev.render_device(st.replace(spp=spp_step, sample_begin=begin + (steps - 1) * spp_step), film.data_ptr(),
                          stream)
        torch.cuda.synchronize()
        a, b = film.double(), mode_film.double()
        out["identical_floats"] = float((film.view(torch.int32) == mode_film.view(torch.int32)).double().mean().item())
        out["relmse_vs_exact"] = float((((b - a) ** 2) / (a ** 2 + 1e-2)).mean().item())
    out["note"] = "; ".join(notes)
    return out


def batch_subrecord(args, rank, world, local, dist):
    """The batched workload (32 scenes, one wavefront per step) for a few steps,
    with the same steps scene by scene on the plain megakernel and on the
    one-scene wavefront: the batched / plain ratio at equal relMSE (every
    renderer gives the same films)."""
    sub = argparse.Namespace(**vars(args))
    sub.steps, sub.warmup, sub.plain_steps, sub.renderer = 4, 3, 1, "auto"
    sub.no_e2e, sub.no_cpu_baseline = True, True
    b = batch_line(sub, rank, world, local, dist)
    plain, seq = b["plain_megakernel"]["value"], b["sequential_wavefront"]["value"]
    return {"value": b["value"], "unit": b["unit"], "steps": sub.steps, "warmup": sub.warmup,
            "ms_per_step": b["ms_per_step"], "plain_megakernel": plain, "vs_plain_megakernel": b["value"] / plain,
            "sequential_wavefront": seq, "vs_sequential_wavefront": b["value"] / seq,
            "autotune": b["run"]["autotune"], "mrays_per_s": b["mrays_per_s"],
            "roofline_frac": b["roofline"]["frac"], "config": b["config"],
            "note": "bench.py --workload batch: 32 scenes as one wavefront (rt_render_batch_device) vs the same "
                    "passes scene by scene (plain megakernel, one-scene wavefront); identical films"}


def adjoint_subrecord(args, rank, world, local, dist):
    """The adjoint workload for a few steps, with its finite-difference checks per
    parameter group (albedo texels, patch alphas)."""
    sub = argparse.Namespace(**vars(args))
    sub.steps, sub.warmup, sub.no_cpu_baseline = 4, 3, True
    a = adjoint_line(sub, rank, world, local, dist)
    return dict(a["adjoint"], steps=sub.steps, warmup=sub.warmup, config=a["config"],
                note="bench.py --workload adjoint: forward + dL/dI + backward per step; fd_check: central finite "
                     "differences with common random numbers per parameter group")


BATCH_STEPS_PER_FRAME = 16


def batch_step_settings(scenes, step):
    """Step `step` of the batched workload: every scene renders the next
    1/16 of its spp (at least 1 sample per pixel)."""
    out = []
    for s, st in scenes:
        spp = max(1, round(st.spp / BATCH_STEPS_PER_FRAME))
        out.append(st.replace(spp=spp, sample_begin=step * spp))
    return out


def batch_config(scenes, step_settings):
    tris = [s.triangle_count for s, _ in scenes]
    return {"workload": f"batch: {len(scenes)} independent scenes (displaced sphere or box, log-uniform "
                        f"{min(tris)}-{max(tris)} triangles, diffuse / GGX conductor / rough dielectric, quad light "
                        "or env), path MIS, rendered as one wavefront (rt_render_batch)",
            "scenes": len(scenes), "triangles": int(sum(tris)),
            "films": sorted({f"{s.camera.width}x{s.camera.height}" for s, _ in scenes}),
            "spp_frame_range": [min(st.spp for _, st in scenes), max(st.spp for _, st in scenes)],
            "max_depth_range": [min(st.max_depth for _, st in scenes), max(st.max_depth for _, st in scenes)],
            "samples_per_step": int(sum(s.camera.width * s.camera.height * st.spp
                                        for (s, _), st in zip(scenes, step_settings))),
            "steps_per_frame": BATCH_STEPS_PER_FRAME}


def run_batch_reference(args):
    """The oracle on a bounded sample of the batch: a centre crop of every 4th scene."""
    from radiantium_gb300 import procedural
    from oracle.oracle import OracleScene
    scenes = procedural.batch_scenes()
    cores = os.cpu_count() or 1
    pick = scenes[::4]
    orcs = [(OracleScene(s), st, s) for s, st in pick]
    crops = []
    for orc, st, s in orcs:
        w, h = min(32, s.camera.width), min(32, s.camera.height)
        crops.append((orc, st.replace(spp=1, x0=(s.camera.width - w) // 2, y0=(s.camera.height - h) // 2,
                                      width=w, height=h), w * h))
    t0 = time.perf_counter()
    for orc, cal, _ in crops:
        orc.render(cal, threads=cores)
    t1 = time.perf_counter() - t0
    spp = int(max(1, (150.0 / (args.steps + args.warmup)) / max(t1, 1e-3)))
    def step(i):
        for orc, cal, _ in crops:
            orc.render(cal.replace(spp=spp, sample_begin=i * spp), threads=cores)
    for i in range(args.warmup):
        step(i)
    times = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        step(args.warmup + i)
        times.append(time.perf_counter() - t0)
    samples = sum(n for _, _, n in crops) * spp
    ms = 1000.0 * float(np.mean(times))
    value = samples / (ms / 1000.0)
    desc = f"centre 32x32 crops of {len(crops)} of the {len(scenes)} scenes x {spp} spp per step ({samples} samples/step)"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scenes)",
        "config": batch_config(scenes, batch_step_settings(scenes, 0)),
        "run": {"step": desc, "parallelism": f"{cores} host threads"},
        "cpu_baseline": {"value": value, "unit": "samples/s", "cores": cores, "kind": "port",
                         "sample": desc + "; the C# reference cannot run here (no .NET), its C++ restatement "
                                          "(oracle/) runs on all host cores"},
        "e2e": {"value": value, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    for orc, _, _ in orcs:
        orc.close()
    print(json.dumps(line), flush=True)
    return 0


def ranks():
    """(rank, world, local rank, torch.distributed or None); joins the NCCL group under torchrun."""
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    return rank, world, local, dist


def run_batch(args):
    rank, world, local, dist = ranks()
    line = batch_line(args, rank, world, local, dist)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def batch_line(args, rank, world, local, dist):
    """The batched workload: 32 scenes rendered as one wavefront per step."""
    import torch
    from radiantium_gb300 import native as N
    from radiantium_gb300 import procedural
    from radiantium_gb300.device import Device

    scenes = procedural.batch_scenes()
    t0 = time.perf_counter()
    devs = []
    for s, _ in scenes:
        d = Device(local)
        d.upload(s)
        devs.append(d)
    upload_s = time.perf_counter() - t0
    host = Device(local)
    mode = N.RENDERER_WAVEFRONT_GRAPH if args.renderer == "graph" else N.RENDERER_WAVEFRONT
    host.set_renderer(mode)
    films = [torch.empty(s.camera.width * s.camera.height * 3, dtype=torch.float32, device="cuda")
             for s, _ in scenes]
    ptrs = [f.data_ptr() for f in films]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    base = rank * (args.warmup + args.steps + 64)

    def items(step):
        return list(zip(devs, batch_step_settings(scenes, base + step)))

    samples_step = sum(s.camera.width * s.camera.height * st.spp
                       for (s, _), st in zip(scenes, batch_step_settings(scenes, 0)))
    tuned = None
    if args.renderer == "auto":
        host.set_renderer(N.RENDERER_AUTO)
        probe = [(d, st.replace(spp=max(1, st.spp // 4), sample_begin=10 ** 6)) for d, st in items(0)]
        tuned = host.autotune(probe)
        mode = N.RENDERER_WAVEFRONT_GRAPH if tuned["renderer"] == N.RENDERER_WAVEFRONT_GRAPH else N.RENDERER_WAVEFRONT
        host.set_renderer(mode)
    host.set_counting(True)
    host.render_batch_device(items(0), ptrs, stream)
    counts = host.stats()
    host.set_counting(False)
    for i in range(args.warmup):
        host.render_batch_device(items(i), ptrs, stream)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    step_ms, loop_ms, shade_ms, launches = [], 0.0, 0.0, 0
    for i in range(args.steps):
        flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        host.render_batch_device(items(args.warmup + i), ptrs, stream)
        e1.record()
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        st = host.stats()
        loop_ms += st["render_kernel_ms"]
        shade_ms += st["shade_kernel_ms"]
        launches += st["kernel_launches"]
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    total_ms = float(np.sum(step_ms))
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / args.steps
    value = samples_step * world / (ms_step / 1000.0)

    e2e = None
    if not args.no_e2e:
        times, h2d = [], []
        for i in range(args.steps):
            t0 = time.perf_counter()
            host.render_batch(items(args.warmup + args.steps + i))
            times.append(time.perf_counter() - t0)
            h2d.append(host.stats()["h2d_bytes"])
        e2e = {"value": samples_step * world / float(np.mean(times)), "unit": "samples/s",
               "h2d_bytes_per_step": int(np.mean(h2d)),
               "d2h_bytes_per_step": int(sum(s.camera.width * s.camera.height * 12 for s, _ in scenes)),
               "note": f"rt_render_batch into host films; scenes resident (32 x rt_upload_scene, {upload_s:.1f} s "
                       "incl. BVH builds)"}

    # the same step scene by scene: plain megakernel, and the one-scene wavefront
    def sequential(renderer):
        for d in devs:
            d.set_renderer(renderer)
        pt = []
        for i in range(max(1, args.plain_steps)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for d, stx, p in zip(devs, batch_step_settings(scenes, base + args.warmup + i), ptrs):
                d.render_device(stx, p, stream)
            e1.record()
            e1.synchronize()
            pt.append(e0.elapsed_time(e1))
        for d in devs:
            d.set_renderer(N.RENDERER_AUTO)
        return samples_step / (float(np.mean(pt)) / 1000.0)

    plain = seq_wf = None
    if args.plain_steps > 0:
        plain = {"value": sequential(N.RENDERER_MEGAKERNEL), "unit": "samples/s", "steps": args.plain_steps,
                 "note": "plain megakernel, the 32 scenes one after another, same passes, identical films"}
        seq_wf = {"value": sequential(N.RENDERER_WAVEFRONT), "unit": "samples/s", "steps": args.plain_steps,
                  "note": "one-scene wavefront (rt_render_device), the 32 scenes one after another"}

    alg_bytes_step = (B_RAY * (counts["rays_closest"] + counts["rays_shadow"]) + B_NODE * counts["node_visits"]
                      + B_PRIM * counts["prim_tests"] + B_INST * counts["instance_visits"] + B_FILM * counts["samples"])
    graph = mode == N.RENDERER_WAVEFRONT_GRAPH
    trace_ms, trace_shade_ms = loop_ms / args.steps, shade_ms / args.steps
    if graph:
        # the graph-driven loop is timed as a whole: the trace kernels' own time comes
        # from one more (untimed) step of the host-driven loop over the same batch
        host.set_renderer(N.RENDERER_WAVEFRONT)
        host.render_batch_device(items(args.warmup), ptrs, stream)
        torch.cuda.synchronize()
        st = host.stats()
        trace_ms, trace_shade_ms = st["render_kernel_ms"], st["shade_kernel_ms"]
        host.set_renderer(mode)
    achieved = alg_bytes_step / (trace_ms / 1000.0) / 1e9
    peak, peak_src = measured_peak()
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_batch(scenes, batch_step_settings(scenes, base), args.cpu_seconds)
    line = {
        "metric": METRIC, "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scenes)",
        "config": batch_config(scenes, batch_step_settings(scenes, 0)),
        "run": {"parallelism": f"replicas x{world} (independent sample passes)",
                "l2": "256 MiB flush between timed steps (outside the CUDA events)",
                "renderer": "batched wavefront, bounce loop as a CUDA graph while-loop" if graph
                else "batched wavefront, bounce loop driven from the host",
                "autotune": tuned},
        "mrays_per_s": (counts["rays_closest"] + counts["rays_shadow"]) * world / (ms_step / 1000.0) / 1e6,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_source": peak_src,
                     "kernel": "k_wf_trace_closest + k_wf_trace_shadow",
                     "kernel_ms_per_step": trace_ms, "shade_ms_per_step": trace_shade_ms,
                     "loop_ms_per_step": loop_ms / args.steps,
                     "note": ("trace / shade times from one step of the host-driven loop" if graph else "")},
        "plain_megakernel": plain,
        "sequential_wavefront": seq_wf,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
        "counts_per_step": {k: counts[k] for k in ("samples", "rays_closest", "rays_shadow", "node_visits",
                                                   "prim_tests", "instance_visits", "invalid_samples")},
    }
    for d in devs:
        d.close()
    host.close()
    return line


def adjoint_setup(d, prm, rng_seed=0):
    """Target film with perturbed albedo (x U[0.7, 1.3]) and alpha (x U[0.7, 1.3])."""
    import math
    s = d.scene
    ti, rts, alpha0 = prm["albedo_texture"], prm["roughness_textures"], prm["alpha"].copy()
    alb0 = s.textures[ti].data.copy()
    rng = np.random.default_rng(rng_seed)

    def set_params(alb, alpha):
        d.update_texture(ti, alb)
        for t, a in zip(rts, alpha):
            d.update_texture(t, np.full(3, math.sqrt(a), np.float32))
    return alb0, alpha0, set_params, (np.clip(alb0 * rng.uniform(0.7, 1.3, alb0.shape), 0.05, 0.95).astype(np.float32),
                                      alpha0 * rng.uniform(0.7, 1.3, alpha0.shape))


def run_adjoint(args):
    rank, world, local, dist = ranks()
    line = adjoint_line(args, rank, world, local, dist)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def adjoint_line(args, rank, world, local, dist):
    """The adjoint workload: one step = forward film + L2-loss gradient + backward
    pass to every albedo texel and every patch alpha."""
    import torch
    from radiantium_gb300 import procedural
    from radiantium_gb300.device import Device
    scene, st, prm = procedural.adjoint_patches()
    d = Device(local)
    d.upload(scene)
    alb0, alpha0, set_params, (alb_t, alpha_t) = adjoint_setup(d, prm)
    set_params(alb_t, alpha_t)
    target = d.render(st.replace(spp=4 * st.spp, seed=99))
    set_params(alb0, alpha0)
    n_params = alb0.size + len(prm["alpha_materials"])
    W, H = scene.camera.width, scene.camera.height
    base = rank * 1000

    def step(i):
        stx = st.replace(seed=base + i)
        img = d.render(stx)
        dl = 2.0 * (img - target)
        ga, gal = d.adjoint_backward(stx, dl, prm["albedo_texture"], prm["alpha_materials"])
        return img, ga, gal

    for i in range(args.warmup):
        step(i)
    d.render(st.replace(seed=base))
    fwd = d.stats()                                  # what a forward render copies and launches (untimed)
    fwd_h2d, fwd_launches = fwd["h2d_bytes"], fwd["kernel_launches"]
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    times, bwd_ms, fwd_times, bwd_h2d, bwd_launches = [], 0.0, [], [], 0
    for i in range(args.steps):
        t0 = time.perf_counter()
        stx = st.replace(seed=base + args.warmup + i)
        img = d.render(stx)
        t1 = time.perf_counter()
        dl = 2.0 * (img - target)
        ga, gal = d.adjoint_backward(stx, dl, prm["albedo_texture"], prm["alpha_materials"])
        times.append(time.perf_counter() - t0)
        fwd_times.append(t1 - t0)
        bwd_ms += d.stats()["render_kernel_ms"]
        bwd_h2d.append(d.stats()["h2d_bytes"])
        bwd_launches += d.stats()["kernel_launches"]
    if dist:
        dist.barrier()
    clk = clocks.stop()
    total_s = float(np.sum(times))
    if dist:
        t = torch.tensor([total_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_s = float(t.item())
    s_step = total_s / args.steps
    samples_step = W * H * st.spp
    fwd_s = float(np.mean(fwd_times))
    # finite-difference checks along one direction per parameter group (linearised loss)
    check = None
    if not args.no_fd_check:
        ref = d.render(st.replace(spp=1024, seed=77))
        w = (2 * (ref - target)).astype(np.float32)
        lin = lambda stx: float((w.astype(np.float64) * d.render(stx)).sum())
        sta = st.replace(seed=3)
        g, _ = d.adjoint_backward(sta, w, prm["albedo_texture"], [])
        v = np.random.default_rng(1).standard_normal(alb0.shape).astype(np.float32)
        set_params(alb0 + 1e-3 * v, alpha0); lp = lin(sta)
        set_params(alb0 - 1e-3 * v, alpha0); lm = lin(sta)
        set_params(alb0, alpha0)
        fd_a, ad_a = (lp - lm) / 2e-3, float((g.reshape(-1).astype(np.float64) * v).sum())
        _, gal = d.adjoint_backward(st.replace(spp=16384, seed=8), w, -1, prm["alpha_materials"])
        va = np.sign(gal) * alpha0
        ad_r = float((gal.astype(np.float64) * va).sum())
        fds = []
        for k in range(8):
            stx = st.replace(spp=4096, seed=100 + k)
            set_params(alb0, alpha0 + 0.01 * va); lp = lin(stx)
            set_params(alb0, alpha0 - 0.01 * va); lm = lin(stx)
            fds.append((lp - lm) / 0.02)
        set_params(alb0, alpha0)
        fd_r = float(np.mean(fds))
        # material by material: the 4 largest |dL/dalpha| (steps of 5 % of that alpha), and one random
        # direction over all alphas (2 % steps); 4 seeds x 4096 spp each
        per = []
        dirs = [(f"material {int(m)}", np.eye(alpha0.size)[m] * alpha0[m], 0.05) for m in np.argsort(-np.abs(gal))[:4]]
        dirs.append(("random", np.random.default_rng(5).standard_normal(alpha0.size) * alpha0, 0.02))
        for name, v, eps in dirs:
            fdk = []
            for k in range(4):
                stx = st.replace(spp=4096, seed=200 + k)
                set_params(alb0, alpha0 + eps * v); lp = lin(stx)
                set_params(alb0, alpha0 - eps * v); lm = lin(stx)
                fdk.append((lp - lm) / (2 * eps))
            set_params(alb0, alpha0)
            fdm, adm = float(np.mean(fdk)), float((gal.astype(np.float64) * v).sum())
            per.append({"direction": name, "fd": fdm, "fd_stderr": float(np.std(fdk, ddof=1) / 2.0),
                        "adjoint": adm, "rel_err": abs(fdm - adm) / abs(fdm)})
        check = {"albedo": {"fd": fd_a, "adjoint": ad_a, "rel_err": abs(fd_a - ad_a) / abs(fd_a),
                            "how": "random normal direction over all texels, eps 1e-3, common random numbers, 64 spp"},
                 "alpha": {"fd": fd_r, "fd_stderr": float(np.std(fds, ddof=1) / math.sqrt(len(fds))), "adjoint": ad_r,
                           "rel_err": abs(fd_r - ad_r) / abs(fd_r),
                           "how": "direction sign(grad) x alpha, eps 1 %, mean of 8 seeds x 4096 spp (common random "
                                  "numbers) vs adjoint at 16384 spp"},
                 "alpha_per_direction": per,
                 "loss": "linearised L2: sum(w * I), w = 2 (I_1024spp - target)"}
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(scene, st, args.cpu_seconds)
        cpu["sample"] = ("forward renders of the oracle (the reference has no derivatives: finite differences "
                         "need two renders per parameter): " + cpu["sample"])
    line = {
        "metric": METRIC, "value": samples_step * world / s_step, "unit": "samples/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * s_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": "adjoint: displaced sphere (one instance, 199,692 triangles) in 64 rough_plastic "
                               "patches sharing a 512x512 albedo texture, Gaussian-lobe env; path MIS; L2 loss "
                               "against a film of perturbed parameters",
                   "film": [W, H], "spp": st.spp, "max_depth": st.max_depth, "parameters": int(n_params),
                   "step": "forward render + dL/dI + backward (gradient w.r.t. all parameters)"},
        "run": {"parallelism": f"replicas x{world}",
                "l2": "inputs resident; no flush (forward and backward re-read the scene)"},
        "adjoint": {"grads_per_s": world / s_step, "params_per_s": n_params * world / s_step,
                    "backward_ms": bwd_ms / args.steps, "forward_ms": 1000.0 * fwd_s,
                    "fd_params_per_s": 1.0 / (2.0 * fwd_s),
                    "vs_fd": (n_params / s_step) / (1.0 / (2.0 * fwd_s)),
                    "fd_check": check},
        "cpu_baseline": cpu,
        "e2e": {"value": samples_step * world / s_step, "unit": "samples/s",
                "h2d_bytes_per_step": int(fwd_h2d + np.mean(bwd_h2d)),
                "d2h_bytes_per_step": W * H * 12 + int(n_params) * 4,
                "note": "the step is timed end to end through the C ABI: film to host, dL/dI from host, gradients to host"},
        "gpu_launches": int(fwd_launches * args.steps + bwd_launches),
        "clocks": clk,
    }
    d.close()
    return line


def particle_workload():
    """The light tracer's workload: the reference's own particle example shape
    (Example/cbox/test_adjoint_particle.json: Cornell box, 800x600, min_depth 7,
    unbounded depth with Russian roulette 0.99), on the procedural Cornell box."""
    from radiantium_gb300 import native as N, procedural
    scene, st = procedural.cornell_box(800, 600)
    return scene, st.replace(integrator=N.INTEGRATOR_PARTICLE, max_depth=-1, min_depth=7, rr_threshold=0.99, seed=1)


def particle_config(scene, st, per_step):
    return {"workload": "adjoint_particle light tracer, procedural Cornell box (36 tris, ceiling quad light), "
                        "min_depth 7, unbounded depth, RR 0.99 (shape of Example/cbox/test_adjoint_particle.json)",
            "film": [scene.camera.width, scene.camera.height], "particles_per_step": per_step,
            "max_depth": st.max_depth, "min_depth": st.min_depth, "integrator": "adjoint_particle",
            "triangles": scene.triangle_count, "seed": st.seed}


def particle_cpu(scene, st, target_s, cores):
    """particles/s of the oracle's light tracer on all host cores, bounded to about target_s."""
    from oracle.oracle import OracleScene
    orc = OracleScene(scene)
    t0 = time.perf_counter()
    orc.render_particles(st, 20000, threads=cores)
    t1 = time.perf_counter() - t0
    n = int(max(20000, min(1 << 26, 20000 * target_s / max(t1, 1e-3))))
    t0 = time.perf_counter()
    orc.render_particles(st, n, first=20000, threads=cores)
    dt = time.perf_counter() - t0
    orc.close()
    return n, dt


def run_particle_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    scene, st = particle_workload()
    cores = os.cpu_count() or 1
    from oracle.oracle import OracleScene
    orc = OracleScene(scene)
    t0 = time.perf_counter()
    orc.render_particles(st, 20000, threads=cores)
    t1 = time.perf_counter() - t0
    total_steps = args.steps + args.warmup
    n = int(max(20000, 20000 * (150.0 / total_steps) / max(t1, 1e-3)))
    for i in range(args.warmup):
        orc.render_particles(st, n, first=i * n, threads=cores)
    times = []
    for i in range(args.steps):
        t0 = time.perf_counter()
        orc.render_particles(st, n, first=(args.warmup + i) * n, threads=cores)
        times.append(time.perf_counter() - t0)
    orc.close()
    ms = 1000.0 * float(np.mean(times))
    value = n / (ms / 1000.0)
    desc = f"{n} particles per step over the whole film (scale + CameraTraceLight included)"
    print(json.dumps({
        "impl": "reference", "metric": "particles/s (adjoint_particle light tracer)", "value": value,
        "unit": "particles/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural scene)", "config": particle_config(scene, st, args.particles_per_step),
        "run": {"step": desc, "parallelism": f"{cores} host threads"},
        "cpu_baseline": {"value": value, "unit": "particles/s", "cores": cores, "kind": "port",
                         "sample": desc + "; the C# reference cannot run here (no .NET), its C++ restatement "
                                          "(oracle/) runs on all host cores"},
        "e2e": {"value": value, "unit": "particles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
        flush=True)
    return 0


def run_particles(args):
    """The light tracer: one step = --particles-per-step particles splatted into the
    whole film, then the film scale and CameraTraceLight pass."""
    import torch
    from radiantium_gb300.device import Device
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from radiantium_gb300 import native as N
    scene, st = particle_workload()
    dev = Device(local)
    dev.upload(scene)
    mode = {"auto": N.RENDERER_AUTO, "megakernel": N.RENDERER_MEGAKERNEL, "wavefront": N.RENDERER_WAVEFRONT,
            "graph": N.RENDERER_WAVEFRONT_GRAPH}[args.renderer]
    dev.set_renderer(mode)
    wavefront = mode != N.RENDERER_MEGAKERNEL
    W, H = scene.camera.width, scene.camera.height
    per = args.particles_per_step
    base = rank * (args.warmup + 2 * args.steps + 1) * per    # disjoint particle ranges per rank
    film = torch.empty(W * H * 3, dtype=torch.float32, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    dev.set_counting(True)
    dev.render_particles_device(st, per, film.data_ptr(), first=base, stream=stream)
    torch.cuda.synchronize()
    counts = dev.stats()
    dev.set_counting(False)
    for i in range(args.warmup):
        dev.render_particles_device(st, per, film.data_ptr(), first=base + (1 + i) * per, stream=stream)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    step_ms, kernel_ms, shade_ms, launches, render_launches = [], 0.0, 0.0, 0, 0
    for i in range(args.steps):
        flush.fill_(float(i))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        dev.render_particles_device(st, per, film.data_ptr(), first=base + (1 + args.warmup + i) * per, stream=stream)
        e1.record()
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        s = dev.stats()
        kernel_ms += s["render_kernel_ms"]
        shade_ms += s["shade_kernel_ms"]
        launches += s["kernel_launches"]
        render_launches += s["render_launches"]
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    total_ms = float(np.sum(step_ms))
    if dist:
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_step = total_ms / args.steps
    value = per * world / (ms_step / 1000.0)
    e2e = None
    if not args.no_e2e:
        import ctypes as C
        host = torch.empty(W * H * 3, dtype=torch.float32, pin_memory=True).numpy()
        p = host.ctypes.data_as(C.c_void_p)
        prm = st.to_c()
        times, h2d = [], []
        for i in range(args.steps):
            t0 = time.perf_counter()
            rc = dev.lib.rt_render_particles(dev.h, C.byref(prm), base + (1 + args.warmup + args.steps + i) * per,
                                             per, p)
            times.append(time.perf_counter() - t0)
            if rc != 0:
                raise RuntimeError(dev.lib.rt_last_error(dev.h).decode())
            h2d.append(dev.stats()["h2d_bytes"])
        e2e = {"value": per * world / float(np.mean(times)), "unit": "particles/s",
               "h2d_bytes_per_step": int(np.mean(h2d)),
               "d2h_bytes_per_step": W * H * 12, "note": "rt_render_particles with a pinned host film"}
    # the one-thread-per-particle megakernel on particle ranges of the same size
    plain = None
    if wavefront and args.plain_steps > 0:
        dev.set_renderer(N.RENDERER_MEGAKERNEL)
        pt = []
        for i in range(args.plain_steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            dev.render_particles_device(st, per, film.data_ptr(), first=base + (1 + args.warmup + i) * per,
                                        stream=stream)
            e1.record()
            e1.synchronize()
            pt.append(e0.elapsed_time(e1))
        dev.set_renderer(mode)
        plain = {"value": per / (float(np.mean(pt)) / 1000.0), "unit": "particles/s", "steps": args.plain_steps,
                 "note": "megakernel k_particles (one thread per particle), same particle ranges"}

    # roofline of the traversal kernels: algorithmic bytes from exact counts (the
    # finishing pass's W*H camera rays are in the counts too; the splats' film
    # atomics are not).  The graph-driven loop is timed as a whole, so the trace
    # kernels' own time comes from one more (untimed) step of the host-driven loop.
    alg = (B_RAY * (counts["rays_closest"] + counts["rays_shadow"]) + B_NODE * counts["node_visits"]
           + B_PRIM * counts["prim_tests"] + B_INST * counts["instance_visits"])
    kms, sms, rls = kernel_ms / args.steps, shade_ms / args.steps, render_launches / args.steps
    if wavefront and mode != N.RENDERER_WAVEFRONT:
        dev.set_renderer(N.RENDERER_WAVEFRONT)
        dev.render_particles_device(st, per, film.data_ptr(), first=base + (1 + args.warmup) * per, stream=stream)
        torch.cuda.synchronize()
        s = dev.stats()
        kms, sms, rls = s["render_kernel_ms"], s["shade_kernel_ms"], s["render_launches"]
        dev.set_renderer(mode)
    achieved = alg / (kms / 1000.0) / 1e9
    peak, peak_src = measured_peak()
    bpp = profiled_traffic("particle", "bytes_per_particle") if wavefront else None
    traffic = None if bpp is None else bpp * per / max(1.0, rls)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cores = os.cpu_count() or 1
        n, dt = particle_cpu(scene, st, args.cpu_seconds, cores)
        cpu = {"value": n / dt, "unit": "particles/s", "cores": cores, "kind": "port",
               "sample": f"{n} particles of the same workload over the whole film ({dt:.1f} s)"}
    line = {
        "metric": "particles/s (adjoint_particle light tracer)", "value": value, "unit": "particles/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded procedural scene)",
        "config": particle_config(scene, st, per),
        "run": {"parallelism": f"replicas x{world} (disjoint particle ranges)",
                "l2": "256 MiB flush between timed steps (outside the CUDA events)",
                "renderer": ("wavefront (trace / shade kernels over compacted queues, particle regeneration)"
                             + (", bounce loop as a CUDA graph" if mode != N.RENDERER_WAVEFRONT else "")
                             if wavefront else "megakernel k_particles (one thread per particle)")
                + " + k_particle_finish"},
        "mrays_per_s": (counts["rays_closest"] + counts["rays_shadow"]) * world / (ms_step / 1000.0) / 1e6,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": traffic, "peak_source": peak_src,
                     "kernel": "k_wf_trace_closest + k_wf_trace_shadow" if wavefront else "k_particles",
                     "alg_bytes_per_step": alg, "kernel_ms_per_step": kms,
                     "launches_per_step": rls, "shade_ms_per_step": sms,
                     "note": ("trace / shade times from one step of the host-driven loop"
                              if wavefront and mode != N.RENDERER_WAVEFRONT else "")},
        "plain_megakernel": plain,
        "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches, "clocks": clk,
        "counts_per_step": {k: counts[k] for k in ("samples", "rays_closest", "rays_shadow", "node_visits",
                                                   "prim_tests", "instance_visits")},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    dev.close()
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.workload == "particle":
        return run_particle_reference(args) if args.impl == "reference" else run_particles(args)
    if args.workload == "adjoint":
        if args.impl == "reference":
            return run_reference(args)
        return run_adjoint(args)
    if args.workload == "batch":
        return run_batch_reference(args) if args.impl == "reference" else run_batch(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
