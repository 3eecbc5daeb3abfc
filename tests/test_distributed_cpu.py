"""Two gloo ranks on CPU render disjoint sample ranges of one frame; the reduced
film equals a single render of the whole range (sample-range sharding)."""
import os
import socket

import numpy as np
import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import torch.distributed as dist

    from oracle import oracle as O
    from pyre_gb300 import presets as P
    from pyre_gb300.distributed import reduce_film_means, sample_range

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc, cam = P.cornell_box(), P.cornell_box_camera(24, 24)
    s0, s1 = sample_range(rank, 4)
    r = O.OracleScene(sc, nthreads=1).render(cam, 24, 24, s1 - s0, spp_begin=s0)
    red = reduce_film_means({"radiance": r["radiance"], "depth": r["depth"]}, s1 - s0)
    if rank == 0:
        np.save(os.path.join(out_dir, "reduced.npy"), red["radiance"])
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sample_sharding(tmp_path, oracle_mod):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    from pyre_gb300 import presets as P
    sc, cam = P.cornell_box(), P.cornell_box_camera(24, 24)
    full = oracle_mod.OracleScene(sc, nthreads=1).render(cam, 24, 24, 8)["radiance"]
    red = np.load(tmp_path / "reduced.npy")
    np.testing.assert_allclose(red, full, rtol=1e-5, atol=1e-6)


def _grad_worker(rank, world, port, out_dir):
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
    import torch.distributed as dist

    from oracle import oracle as O
    from pyre_gb300 import presets as P
    from pyre_gb300.distributed import reduce_gradients

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc, cam = P.studio_ref(), P.studio_ref_camera(16, 16)
    dl = np.random.default_rng(5).normal(size=(16, 16, 3)).astype(np.float32)
    env_shape = (sc.env.height, sc.env.width)
    s0, s1 = (0, 2) if rank == 0 else (2, 6)  # uneven sample ranges
    mat, env = O.OracleScene(sc, nthreads=1).render_grad(cam, 16, 16, s1 - s0, dl, len(sc.materials), env_shape,
                                                         spp_begin=s0, max_depth=5)
    rm, re = reduce_gradients(mat, env, s1 - s0)
    if rank == 0:
        np.save(os.path.join(out_dir, "mat.npy"), rm)
        np.save(os.path.join(out_dir, "env.npy"), re)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gradient_reduction(tmp_path, oracle_mod):
    """Ranks differentiate disjoint sample ranges of unequal length ([0,2) and
    [2,6)); the count-weighted all-reduce equals the gradient of the whole range."""
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_grad_worker, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    from pyre_gb300 import presets as P
    sc, cam = P.studio_ref(), P.studio_ref_camera(16, 16)
    dl = np.random.default_rng(5).normal(size=(16, 16, 3)).astype(np.float32)
    mat, env = oracle_mod.OracleScene(sc, nthreads=1).render_grad(cam, 16, 16, 6, dl, len(sc.materials),
                                                                  (sc.env.height, sc.env.width), max_depth=5)
    rm, re = np.load(tmp_path / "mat.npy"), np.load(tmp_path / "env.npy")
    assert np.abs(mat).max() > 0 and np.abs(env).max() > 0
    # Each path term is scaled by 1/spp in f32, so the split ranges round differently.
    np.testing.assert_allclose(rm, mat, rtol=1e-5, atol=1e-7 * np.abs(mat).max())
    np.testing.assert_allclose(re, env, rtol=1e-5, atol=1e-6 * np.abs(env).max())
