"""The continuous-batching server (mcrt_server_*): results equal simulate(), a request's
result is the same alone and in a mix, admission respects the memory cap, and graph
replay equals direct launches."""
import json
import math
import time

import numpy as np
import pytest

from helpers import scaled_err

pytestmark = pytest.mark.gpu
N0 = [1.0, 0.0, 0.0, 0.0]


def small_cfg(M, g):
    return M.Config(g, number_of_rays=1, Ntheta=16, Nphi=8, Nphib=4, thetab=np.deg2rad(np.linspace(0, 3, 12)),
                    maximum_scattering_times=400)


def requests(M, mie5, mie2):
    ray = M.RayleighScatterer(0.97, 100.0)
    out = []
    for i in range(12):
        if i % 3 == 0:
            g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=(0.5 + i) * ray.kl, scatterer=ray)])
        elif i % 3 == 1:
            g = M.PlaneGeometry(math.radians(140 + i), 0.2 * i, [M.Layer(d=(0.3 + 0.2 * i) * mie5.kl, scatterer=mie5)])
        else:
            g = M.SphereGeometry(R=(1 + 0.3 * i) * mie2.kl, scatterer=mie2)
        I = [N0, [1, 1, 0, 0], [1, 0, 0, -1]][i % 3]
        out.append((small_cfg(M, g), g, I, 200 + 377 * i, 100 + i, i))
    return out


def compare(a, b, tol):
    assert scaled_err(a[0], b[0]) < tol
    assert scaled_err(a[1], b[1]) < tol
    assert scaled_err(a[2], b[2]) < tol


def test_server_results_match_simulate(M, gpu_ctx, mie5, mie2, tmp_path):
    reqs = requests(M, mie5, mie2)[:6]
    log = tmp_path / "serve.jsonl"
    srv = M.Server(precision="fp64", wave_photons=2048, min_quantum=256, log_path=str(log))
    t0 = time.perf_counter()
    tickets = [srv.submit(c, g, I, n, seed=s, instance=i) for c, g, I, n, s, i in reqs]
    for t, (c, g, I, n, s, i) in zip(tickets, reqs):
        A, Irt, Icb, lad, info = srv.result(t)
        solo = M.simulate(c.replace(number_of_rays=n), g, I, precision="fp64", seed=s, instance=i)
        compare((A, Irt, Icb), (np.array(solo[:5]), solo[5], solo[6]), 1e-9)
        assert info["photons"] == n and info["waves"] >= 1
        assert info["submitted_s"] <= info["admitted_s"] <= info["completed_s"]
    wall = time.perf_counter() - t0
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["resident_bytes"] == 0
    # waves overlap on two streams; busy time is the union of their intervals
    assert 0 < st["busy_s"] <= wall
    srv.close()
    lines = [json.loads(x) for x in log.read_text(encoding="utf-8").splitlines()]
    assert len(lines) == len(reqs) and all(x["latency_s"] >= x["queued_s"] >= 0 for x in lines)


@pytest.mark.parametrize("quanta", ["work", "photons"])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("fp32", 1e-4)])
def test_result_is_the_same_alone_and_in_the_mix(M, gpu_ctx, mie5, mie2, prec, tol, quanta):
    """Waves sized in bin evaluations (each request's quantum from its measured cost per
    photon) and in photons: small waves, so that the request's photons are spread over
    several waves shared with the others."""
    reqs = requests(M, mie5, mie2)
    x = reqs[4]
    if quanta == "work":
        srv = M.Server(precision=prec, wave_work=2e7)
    else:
        srv = M.Server(precision=prec, wave_photons=4096, min_quantum=512)
    c, g, I, n, s, i = x
    alone = srv.result(srv.submit(c, g, I, 4 * n, seed=s, instance=i))
    tickets = []
    for k, (c2, g2, I2, n2, s2, i2) in enumerate(reqs):
        if k == 4:
            tickets.append(srv.submit(c, g, I, 4 * n, seed=s, instance=i))
        else:
            tickets.append(srv.submit(c2, g2, I2, n2, seed=s2, instance=i2))
    mixed = srv.result(tickets[4])
    for k, t in enumerate(tickets):
        if k != 4:
            srv.result(t)
    compare(mixed[:3], alone[:3], tol)
    assert mixed[4]["waves"] >= 2  # its photons were spread over waves shared with others
    srv.close()


def test_admission_respects_the_memory_cap_and_waits_time_out(M, gpu_ctx, mie5, mie2):
    reqs = requests(M, mie5, mie2)
    srv0 = M.Server(precision="fp32")
    t0 = srv0.submit(*reqs[0][:4])
    fp = srv0.result(t0)[4]["footprint_bytes"]
    srv0.close()
    cap = 2.5 * fp
    srv = M.Server(precision="fp32", memory_cap_bytes=cap, wave_photons=2048, min_quantum=256)
    ts = [srv.submit(c, g, I, n, seed=s, instance=i) for c, g, I, n, s, i in reqs[:6:3] * 3]
    big = srv.submit(*reqs[0][:3], 200000)
    assert srv.wait(big, 0.001) is False  # still queued or running
    for t in ts:
        srv.result(t)
    srv.result(big)
    st = srv.stats()
    assert st["peak_resident_bytes"] <= cap
    assert st["completed"] == len(ts) + 1
    srv.close()


def test_graph_replay_matches_direct_launches(M, gpu_ctx, mie5, mie2):
    reqs = requests(M, mie5, mie2)[1:4]
    outs = []
    for graphs in (True, False):
        srv = M.Server(precision="fp64", use_graphs=graphs, wave_photons=2048, min_quantum=256)
        ts = [srv.submit(c, g, I, n, seed=s, instance=i) for c, g, I, n, s, i in reqs]
        outs.append([srv.result(t) for t in ts])
        srv.close()
    for a, b in zip(*outs):
        compare(a[:3], b[:3], 1e-9)


def test_requests_with_device_made_mie_tables(M, gpu_ctx):
    """A serving stream whose requests bring new (x, m): the tables are made on the device
    in one launch (mcrt_mie_scatterers_create) and the requests run on them; each result
    equals simulate() with the same device-made scatterer."""
    rng = np.random.default_rng(11)
    params = [(float(x) / (2 * math.pi), complex(rng.uniform(1.3, 1.6), 10 ** rng.uniform(-5, -2)), 1.0, 0.1)
              for x in rng.uniform(0.5, 10.0, 4)]
    scats = gpu_ctx.mie_scatterers(params, Ntheta=721)
    srv = M.Server(ctx=gpu_ctx, precision="fp64", wave_photons=2048, min_quantum=256)
    reqs = []
    for i, sc in enumerate(scats):
        g = M.PlaneGeometry(math.radians(150 + 5 * i), 0.1 * i, [M.Layer(d=(0.5 + i) * sc.kl, scatterer=sc)])
        reqs.append((small_cfg(M, g), g, 300 + 200 * i, 50 + i))
    tickets = [srv.submit(c, g, N0, n, seed=s, instance=0) for c, g, n, s in reqs]
    for t, (c, g, n, s) in zip(tickets, reqs):
        A, Irt, Icb, lad, info = srv.result(t)
        solo = M.simulate(c.replace(number_of_rays=n), g, N0, ctx=gpu_ctx, precision="fp64", seed=s, instance=0)
        compare((A, Irt, Icb), (np.array(solo[:5]), solo[5], solo[6]), 1e-9)
    srv.close()
