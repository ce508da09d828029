"""One film on several GPUs: replicas with no data-path collective.

Camera samples are independent, so N ranks (one process per GPU) split the
film's sample indices into contiguous ranges, each renders its range of the
same film (`sample_begin`), and the films are combined once at the end: the
spp-weighted sum of the rank films, reduced over the ranks, divided by the
total spp (BlockBasedRenderer's per-pixel average).  The combined film
equals the one-GPU film up to the order of the final float additions.

The light tracer shards the same way over particle ranges: particle i's
random numbers depend only on (seed, i), and each rank's film is already its
splats scaled by 1/(its particle count) plus CameraTraceLight, so the
count-weighted mean of the rank films is the film of all the particles.
"""
from __future__ import annotations

import numpy as np


def sample_range(rank: int, world: int, spp: int) -> tuple[int, int]:
    """(first sample index, count) of `rank`: contiguous, disjoint, covering [0, spp)."""
    if world < 1 or not 0 <= rank < world or spp < 0:
        raise ValueError("bad rank / world / spp")
    base, extra = divmod(spp, world)
    return rank * base + min(rank, extra), base + (1 if rank < extra else 0)


def combine(film: np.ndarray, count: int, total: int, group=None) -> np.ndarray:
    """Average of the rank films weighted by their sample counts (float64 sum,
    one all-reduce), returned on every rank."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.asarray(film, dtype=np.float64) * float(count))
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return (t.numpy() / float(total)).astype(np.float32)


def render_replicated(render, settings, rank: int, world: int, group=None) -> np.ndarray:
    """render(settings) -> film of this rank's sample range; returns the combined film."""
    begin, count = sample_range(rank, world, settings.spp)
    if count == 0:
        film = None
    else:
        film = render(settings.replace(spp=count, sample_begin=settings.sample_begin + begin))
    if film is None:
        probe = render(settings.replace(spp=1))
        film = np.zeros_like(probe)
    return combine(film, count, settings.spp, group)


def render_particles_replicated(render_particles, settings, count: int, rank: int, world: int,
                                group=None) -> np.ndarray:
    """render_particles(settings, n, first) -> film of particles [first, first + n) (the
    light tracer, "adjoint_particle"); returns the film of particles [0, count)."""
    if count < 1:
        raise ValueError("particle count must be >= 1")
    first, n = sample_range(rank, world, count)
    film = render_particles(settings, n, first) if n > 0 else None
    if film is None:
        film = np.zeros_like(render_particles(settings, 1, 0))
    return combine(film, n, count, group)
