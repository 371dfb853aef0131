"""The multi-GPU form shards photon index ranges across ranks (counter-based streams
make every photon independent of where it runs) and sums the tallies once at the end.
Covered here on CPU with world_size 2 over gloo, using the oracle as each rank's
transport; the only exchange is the final all-reduce."""
import math
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _config():
    sys.path.insert(0, os.path.join(ROOT, "montecarloradiativetransfer.jl_gb300"))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import mcrt_gb300 as M

    ray = M.RayleighScatterer(0.99, 100.0)
    g = M.PlaneGeometry(math.radians(160), 0.0, [M.Layer(d=3 * ray.kl, scatterer=ray)])
    cfg = M.Config(g, number_of_rays=400, Ntheta=16, Nphi=8, Nphib=4,
                   thetab=np.deg2rad(np.linspace(0, 2, 8)), maximum_scattering_times=300)
    return cfg, g


def _worker(rank, world, port, outdir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle as O

    cfg, g = _config()
    n = cfg.number_of_rays // world
    r = O.simulate(cfg, g, [1, 0, 0, 0], seed=8, threads=1, photon_begin=rank * n, photon_count=n)
    flat = torch.tensor(np.concatenate([r["A"], r["Irt"].ravel(), r["Icb"].ravel()]), dtype=torch.float64)
    dist.all_reduce(flat)
    if rank == 0:
        np.save(os.path.join(outdir, "sharded.npy"), flat.numpy())
    dist.destroy_process_group()


def test_photon_sharding_over_two_ranks_equals_one_run(tmp_path):
    from helpers import free_port

    port = free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    sharded = np.load(tmp_path / "sharded.npy")
    import oracle as O

    cfg, g = _config()
    r = O.simulate(cfg, g, [1, 0, 0, 0], seed=8, threads=1)
    whole = np.concatenate([r["A"], r["Irt"].ravel(), r["Icb"].ravel()])
    assert np.max(np.abs(sharded - whole)) <= 1e-12 * np.max(np.abs(whole))
