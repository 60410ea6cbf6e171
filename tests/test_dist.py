"""Multi-rank host logic on the CPU (gloo, world size 2): sample-range
sharding and the film reduction.  Each rank renders its share of the
samples with the oracle (the GPU path needs a GPU per rank; the split and
the reduction are the same code); rank 0 checks the merged film against one
process rendering every sample."""
import os
import socket

import numpy as np
import pytest

from eleven import dist as D

torch = pytest.importorskip("torch")


def test_shard_samples_cover_the_range_once():
    for spp in (0, 1, 7, 64, 65):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                first, n = D.shard_samples(spp, r, world, sample_begin=5)
                seen.extend(range(first, first + n))
            assert seen == list(range(5, 5 + spp))
    with pytest.raises(ValueError):
        D.shard_samples(4, 2, 2)


def test_merge_films_weights_by_samples():
    a = np.ones((3, 4), np.float32)
    b = np.ones((3, 4), np.float32)
    a[:, :3] = 1.0
    b[:, :3] = 4.0
    out, cnt = D.merge_films([a, b], [np.array([1, 3, 0]), np.array([3, 1, 0])])
    np.testing.assert_allclose(out[:, 0], [3.25, 1.75, 0.0])
    assert (out[:, 3] == 1).all()
    np.testing.assert_array_equal(cnt, [4, 4, 0])


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    sys.path.insert(0, os.path.join(os.path.dirname(here), "tfg-pathtracer_gb300"))
    import torch.distributed as dist
    import _oracle as O
    from eleven import dist as DD
    from eleven import scenes
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        arrays = scenes.config0(x_res=24, y_res=16, n_spheres=4, subdiv=1)
        orc = O.OrcScene(arrays)
        first, n = DD.shard_samples(6, rank, world)
        out = orc.render(spp=n, max_depth=3, seed=4, sample_begin=first)
        beauty, samples = DD.reduce_film(out["beauty"], out["samples"])
        # the exact form: FP64 sums (here the share's mean times its counts)
        own = out["beauty"][:, :3].astype(np.float64) * out["samples"][:, None]
        sums, cnt, b2 = DD.reduce_sums(own, out["samples"])
        if rank == 0:
            q.put((beauty, samples, sums, cnt, b2))
        orc.close()
    finally:
        dist.destroy_process_group()


def test_two_ranks_merge_to_the_single_process_film():
    import torch.multiprocessing as mp
    sys_path = os.path.dirname(os.path.abspath(__file__))
    import sys
    sys.path.insert(0, sys_path)
    import _oracle as O
    from eleven import scenes
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    beauty, samples, sums, cnt, b2 = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    arrays = scenes.config0(x_res=24, y_res=16, n_spheres=4, subdiv=1)
    orc = O.OrcScene(arrays)
    ref = orc.render(spp=6, max_depth=3, seed=4)
    orc.close()
    np.testing.assert_array_equal(samples, ref["samples"])
    # the reference's FP32 running mean against a float64 weighted mean of
    # two FP32 running means: equal up to float rounding
    np.testing.assert_allclose(beauty[:, :3], ref["beauty"][:, :3], rtol=2e-5, atol=1e-6)
    assert (beauty[:, 3] == 1).all()
    # reduce_sums: the ranks' sums added, the merged mean rounded once
    orc = O.OrcScene(arrays)
    parts = [orc.render(spp=3, max_depth=3, seed=4, sample_begin=b) for b in (0, 3)]
    orc.close()
    want = sum(p["beauty"][:, :3].astype(np.float64) * p["samples"][:, None] for p in parts)
    np.testing.assert_allclose(sums, want, rtol=1e-15, atol=0)
    np.testing.assert_array_equal(cnt, ref["samples"])
    np.testing.assert_array_equal(b2[:, :3], (want / np.maximum(cnt, 1)[:, None]).astype(np.float32))
