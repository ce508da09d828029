"""Replica sharding of one film over ranks (radiantium_gb300.replicas), run as
world_size-2 gloo process groups on the CPU with the oracle as each rank's
renderer: the combined film equals the one-process film to float rounding."""
import os

import numpy as np
import pytest

from radiantium_gb300.replicas import sample_range


@pytest.mark.parametrize("world,spp", [(1, 7), (2, 8), (2, 7), (3, 2), (4, 9)])
def test_sample_ranges_partition(world, spp):
    got = [sample_range(r, world, spp) for r in range(world)]
    idx = [i for b, c in got for i in range(b, b + c)]
    assert idx == list(range(spp))
    assert max(c for _, c in got) - min(c for _, c in got) <= 1


def _rank_main(rank, world, port, path):
    import torch.distributed as dist
    from oracle.oracle import OracleScene
    from radiantium_gb300 import procedural
    from radiantium_gb300.replicas import render_replicated
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s, st = procedural.cornell_box(64, 64)
    orc = OracleScene(s)
    st = st.replace(x0=20, y0=20, width=12, height=10, spp=7, seed=3)
    film = render_replicated(lambda x: orc.render(x, threads=2), st, rank, world)
    np.save(os.path.join(path, f"rank{rank}.npy"), film)
    dist.barrier()
    dist.destroy_process_group()
    orc.close()


def test_two_gloo_ranks_combine_to_the_single_film(tmp_path):
    import socket
    import torch.multiprocessing as mp
    from oracle.oracle import OracleScene
    from radiantium_gb300 import procedural
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    s, st = procedural.cornell_box(64, 64)
    one = OracleScene(s).render(st.replace(x0=20, y0=20, width=12, height=10, spp=7, seed=3))
    a, b = np.load(tmp_path / "rank0.npy"), np.load(tmp_path / "rank1.npy")
    assert np.array_equal(a, b)
    assert np.allclose(a, one, rtol=2e-6, atol=1e-7)


def _particle_rank_main(rank, world, port, path):
    import torch.distributed as dist
    from oracle.oracle import OracleScene
    from radiantium_gb300 import native as N, procedural
    from radiantium_gb300.replicas import render_particles_replicated
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    s, st = procedural.cornell_box(24, 20)
    orc = OracleScene(s)
    pst = st.replace(integrator=N.INTEGRATOR_PARTICLE, seed=5)
    film = render_particles_replicated(lambda x, n, f: orc.render_particles(x, n, first=f, threads=2), pst, 30001,
                                       rank, world)
    np.save(os.path.join(path, f"prank{rank}.npy"), film)
    dist.barrier()
    dist.destroy_process_group()
    orc.close()


def test_two_gloo_ranks_combine_particle_films(tmp_path):
    """Light tracer: two ranks each trace half of the particle range; the combined film
    equals the one-process film of the whole range to float rounding."""
    import socket
    import torch.multiprocessing as mp
    from oracle.oracle import OracleScene
    from radiantium_gb300 import native as N, procedural
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    mp.start_processes(_particle_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    s, st = procedural.cornell_box(24, 20)
    one = OracleScene(s).render_particles(st.replace(integrator=N.INTEGRATOR_PARTICLE, seed=5), 30001)
    a, b = np.load(tmp_path / "prank0.npy"), np.load(tmp_path / "prank1.npy")
    assert np.array_equal(a, b)
    assert np.allclose(a, one, rtol=1e-5, atol=1e-6 * float(one.max()))
