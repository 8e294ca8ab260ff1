"""Host logic of multi-GPU rendering (muon_gb300/replicas.py) on CPU: sample
ranges of the ranks, and the film merge and step reductions run as two gloo
ranks in separate processes."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from muon_gb300 import replicas


@pytest.mark.parametrize("world", [1, 2, 3, 8])
@pytest.mark.parametrize("spp", [0, 1, 7, 64, 1000])
def test_sample_ranges_cover_every_sample_once(world, spp):
    seen = []
    for rank in range(world):
        off, n = replicas.sample_range(rank, world, spp)
        seen += list(range(off, off + n))
    assert seen == list(range(spp))
    counts = [replicas.sample_range(r, world, spp)[1] for r in range(world)]
    assert max(counts) - min(counts) <= 1


def test_sample_range_rejects_bad_arguments():
    for args in [(0, 0, 4), (2, 2, 4), (-1, 2, 4), (0, 2, -1)]:
        with pytest.raises(ValueError):
            replicas.sample_range(*args)


def _film(rank, h=5, w=7):
    rng = np.random.default_rng(100 + rank)
    return (rng.random((h, w, 3)), rng.random((h, w, 3)), rng.integers(0, 50, (h, w)).astype(np.int32))


def _rank_main(rank, world, port, out_dir):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        s, q, c = (torch.from_numpy(a.copy()) for a in _film(rank))
        replicas.merge_films(s, q, c)
        ms, counted = replicas.reduce_step(10.0 + rank, 1000 * (rank + 1))
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), s=s.numpy(), q=q.numpy(), c=c.numpy(),
                 ms=ms, counted=counted)
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return sk.getsockname()[1]


def test_two_ranks_merge_films_and_reduce_steps(tmp_path):
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    films = [_film(r) for r in range(world)]
    want_s = sum(f[0] for f in films)
    want_q = sum(f[1] for f in films)
    want_c = sum(f[2] for f in films)
    for rank in range(world):
        got = np.load(tmp_path / f"rank{rank}.npz")
        np.testing.assert_allclose(got["s"], want_s, rtol=1e-15)
        np.testing.assert_allclose(got["q"], want_q, rtol=1e-15)
        assert np.array_equal(got["c"], want_c)
        assert float(got["ms"]) == 11.0            # the slowest rank
        assert float(got["counted"]) == 3000.0     # rays of all ranks


def test_reduce_step_without_a_process_group():
    assert replicas.reduce_step(3.5, 42) == (3.5, 42.0)
