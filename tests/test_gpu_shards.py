"""Photon sharding across processes through the library: two gloo ranks on one GPU each
run their own photon index range with libmcrt (counter-based Philox streams make a
photon's path independent of the rank that runs it), then sum their raw tallies with one
all-reduce, the only exchange the sharded form has. The sum must equal one run of all
the photons. The ranks' kernels never wait on each other; the all-reduce is on host
tensors after each rank's launch has finished."""
import math
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

pytestmark = pytest.mark.gpu
N_PHOTONS = 6000


def _workload(M, O):
    from conftest import oracle_made_mie

    mie = oracle_made_mie(M, O, 5.0, 1.5 + 0.001j)
    g = M.PlaneGeometry(math.radians(150), 0.3, [M.Layer(d=2.0 * mie.kl, scatterer=mie)])
    cfg = M.Config(g, number_of_rays=N_PHOTONS, Ntheta=16, Nphi=8, Nphib=4,
                   thetab=np.deg2rad(np.linspace(0, 3, 12)), maximum_scattering_times=500)
    return cfg, g


def _raw(r):
    return np.concatenate([r["A"], r["Irt"].ravel(), r["Icb"].ravel(), r["ladder"].ravel()])


def _rank(rank, world, port, outdir, prec):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import mcrt_gb300 as M
    import oracle as O

    cfg, g = _workload(M, O)
    n = N_PHOTONS // world
    begin = rank * n
    count = N_PHOTONS - begin if rank == world - 1 else n
    s = M.Solve(cfg, g, [1, 0, 1, 0], precision=prec, seed=23)
    s.launch(begin, count)
    r = s.read()
    s.close()
    np.save(os.path.join(outdir, f"rank{rank}_{prec}.npy"), np.array([begin, count, r["stats"]["photons"]]))
    flat = torch.from_numpy(_raw(r).copy())
    dist.all_reduce(flat)
    if rank == 0:
        np.save(os.path.join(outdir, f"sharded_{prec}.npy"), flat.numpy())
    dist.destroy_process_group()


# FP64 lanes keep FP64 partial sums, so the shards' sum equals one run to rounding. FP32
# lanes sum a batch of events in FP32 before their FP64 flush, and which photons share a
# batch depends on the launch, so the FP32 sums agree to the FP32 partials' rounding.
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_library_photon_shards_over_two_ranks_sum_to_one_run(M, O, gpu_ctx, tmp_path, prec, tol):
    from helpers import free_port

    port = free_port()
    mp.spawn(_rank, args=(2, port, str(tmp_path), prec), nprocs=2, join=True)
    sharded = np.load(tmp_path / f"sharded_{prec}.npy")
    ranks = [np.load(tmp_path / f"rank{k}_{prec}.npy").tolist() for k in range(2)]
    for begin, count, photons in ranks:  # each rank ran exactly its own range
        assert photons == count, ranks
    cfg, g = _workload(M, O)
    s = M.Solve(cfg, g, [1, 0, 1, 0], precision=prec, seed=23)
    s.launch(0, N_PHOTONS)
    whole = _raw(s.read())
    s.close()
    assert whole[5:].any()
    assert np.max(np.abs(sharded - whole)) <= tol * np.max(np.abs(whole))


def _first_launch(rank, prec, outdir):
    import mcrt_gb300 as M
    import oracle as O

    cfg, g = _workload(M, O)
    out = []
    for trial in range(3):
        s = M.Solve(cfg, g, [1, 0, 1, 0], precision=prec, seed=23 + trial)
        begin = 3000 * rank
        s.launch(begin, 3000)  # the first launch asks for a range other than the solve's own
        out.append(s.read()["stats"]["photons"])
        s.close()
    np.save(os.path.join(outdir, f"first_{rank}_{prec}.npy"), np.array(out))


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_first_launch_runs_its_range_while_another_process_shares_the_gpu(gpu_ctx, tmp_path, prec):
    """Two processes create solves and launch at once on one GPU. Each solve's first launch
    asks for a photon range other than the one the solve was created with; its instance
    update must not be overtaken by the creation-time upload (a stale copy landing last
    made such a launch run all 6 000 photons)."""
    mp.spawn(_first_launch, args=(prec, str(tmp_path)), nprocs=2, join=True)
    for rank in range(2):
        got = np.load(tmp_path / f"first_{rank}_{prec}.npy")
        assert np.all(got == 3000), (rank, got)
