#!/usr/bin/env python
"""Photon paths/s of the polarised Monte Carlo transport with coherent backscattering.

Workload (one GPU): Mie spheres of size parameter 5 and refractive index 1.5+0.001i
(1801-angle tables stored in FP32), a plane slab of optical thickness 5 with the Mie
albedo, incidence zenith angle 30 degrees, unpolarised light, the reference's default
bin grids, FP32 transport with FP64 CB phase reduction and FP64 tallies. One step is
one persistent launch over a batch of photons (2^22 by default); the workload's full
size is 1e8 photons, and the line's config states the photons actually timed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line. ``value`` is device-timed throughput with the inputs resident;
``e2e`` is the same metric through the C ABI call mcrt_simulate with host buffers.
With N > 1 (torchrun, one rank per GPU) the photon ranges are sharded across ranks
with no collective in the data path (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "montecarloradiativetransfer.jl_gb300"))

WORKLOAD = "mie_x5_m1.5+0.001i_slab_tau5_zenith30"
FULL_WORKLOAD_PHOTONS = 100_000_000  # the workload's stated size; the line reports what was timed
# Algorithmic flops per bin evaluation of the reference's algorithm for a Mie
# scatterer: additions + multiplications (FMA = 2), special functions (div, sqrt, exp,
# sin/cos, acos) not counted. They come from the oracle's per-bin arithmetic
# instantiated with an operation-counting scalar (oracle/opcount.cpp), and
# tests/test_opcount.py checks these constants against it. Per RT peel-off bin, CB
# reciprocal-path bin and CB single-scattering bin.
FLOPS_RT_MIE = 128.349
FLOPS_CBN_MIE = 409.0
FLOPS_CB1_MIE = 196.0
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one transport launch
# per photon, from an ncu capture of `bench.py --case 524288` (3.77 MB read + 1.214 GB
# written for 524 288 photons). The traffic is dirty L2 lines of the per-event
# photon-state pool and of the threads' spill slots written back; it scales with the
# photons' events, so a full launch is this times its photons.
NCU_DRAM_BYTES_PER_PHOTON = 2321.9


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=1 << 22, help="photons per step per GPU")
    ap.add_argument("--fp64-sample", type=int, default=1 << 16)
    ap.add_argument("--cpu-sample", type=int, default=2000,
                    help="photons per step of the reference arm (and its warm-up, a quarter)")
    ap.add_argument("--cpu-baseline-sample", type=int, default=20000,
                    help="photons of the GPU arm's cpu_baseline leg: about 15 s on 16 host cores")
    ap.add_argument("--no-extras", action="store_true", help="skip the FP64, CPU and serving legs")
    ap.add_argument("--case", type=int, default=0,
                    help="run one FP32 launch of the workload with this many photons and exit "
                         "(the small case for ncu captures)")
    ap.add_argument("--case-precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--case-workload", default="mie_slab", choices=["mie_slab", "rayleigh_slab", "mie_sphere"],
                    help="workload of --case: the Mie slab, the Rayleigh slab (tau 10, Ntheta 180, 200 "
                         "CB angles) or the Mie sphere (tau 20, x 2, 500 CB angles)")
    ap.add_argument("--serve-requests", type=int, default=4096)
    ap.add_argument("--serve-scale", type=float, default=1e-3, help="photon budget multiplier of the stream")
    return ap.parse_args()


def workload(M, n_rays):
    mie = M.MieScatterer(5.0 / (2 * math.pi), 1.5 + 0.001j, 1.0, 0.1, Ntheta=1801)
    g = M.PlaneGeometry(math.radians(150.0), 0.0, [M.Layer(d=5.0 * mie.kl, scatterer=mie)])
    cfg = M.Config(g, number_of_rays=n_rays)
    return mie, g, cfg


class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [s.strip() for s in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        top = max(sm)
        loaded = [s for s in sm if s >= 0.5 * top] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def serve_leg(M, ctx, n_req, scale, rate_hz=200.0, seed=5):
    """The serving stream: Poisson arrivals at rate_hz of requests drawn like the
    4096-request mix (plane 70% / sphere 30%, optical size log-uniform in [0.1, 50],
    albedo uniform in [0.5, 0.9999], Rayleigh or Mie with x in U[0.5, 10], n in
    U[1.3, 1.6], k log-uniform in [1e-5, 1e-2] on 1801 angles, photon budgets
    log-uniform in [1e4, 1e7]) with the budgets multiplied by `scale` so the stream
    fits a short run; admission cap 20 GB."""
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n_req):
        if rng.random() < 0.5:
            sc = M.RayleighScatterer(rng.uniform(0.5, 0.9999), 1.0)
        else:
            x = rng.uniform(0.5, 10.0)
            m = complex(rng.uniform(1.3, 1.6), 10 ** rng.uniform(-5, -2))
            sc = M.MieScatterer(x / (2 * math.pi), m, 1.0, 0.1, Ntheta=1801)
        size = 10 ** rng.uniform(-1, math.log10(50))
        omega = rng.uniform(0.5, 0.9999)
        if rng.random() < 0.7:
            g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=size * sc.kl, scatterer=sc, omega=omega)])
        else:
            g = M.SphereGeometry(R=size * sc.kl, scatterer=sc, omega=omega)
        n = max(1, int(round(10 ** rng.uniform(4, 7) * scale)))
        reqs.append((M.Config(g, number_of_rays=n), g, n))
    srv = M.Server(ctx=ctx, memory_cap_bytes=20e9, precision="fp32")
    arrivals = np.cumsum(rng.exponential(1.0 / rate_hz, n_req))
    t0 = time.perf_counter()
    tickets = []
    for k, (cfg, g, n) in enumerate(reqs):
        delay = arrivals[k] - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        tickets.append(srv.submit(cfg, g, [1.0, 0.0, 0.0, 0.0], n, seed=seed, instance=k))
    lat, first, last, photons = [], math.inf, 0.0, 0
    for t, (cfg, g, n) in zip(tickets, reqs):
        info = srv.result(t)[4]
        lat.append(info["completed_s"] - info["submitted_s"])
        first = min(first, info["submitted_s"])
        last = max(last, info["completed_s"])
        photons += n
    st = srv.stats()
    srv.close()
    lat = np.array(lat)
    return {"requests": n_req, "arrival_rate_hz": rate_hz, "budget_scale": scale,
            "p50_latency_s": float(np.percentile(lat, 50)), "p99_latency_s": float(np.percentile(lat, 99)),
            "paths_per_s": photons / (last - first), "photons": photons, "waves": st["waves"],
            "gpu_busy_s": st["busy_s"], "peak_resident_bytes": st["peak_resident_bytes"],
            "memory_cap_bytes": 20e9}


def batch_leg(M, ctx, n_inst=256, scale=1.5e-2, seed=4):
    """One persistent launch over uneven slab instances drawn like the 256-instance batch
    (optical thickness log-uniform in [0.1, 50], albedo uniform in [0.5, 0.9999], Rayleigh
    or Mie with x in U[0.5, 10], n in U[1.3, 1.6], k log-uniform in [1e-5, 1e-2] on 1801
    angles, photon budgets lognormal(median 1e7, sigma 1)) with the budgets multiplied by
    `scale` (1.5e-2: 5.7e7 paths for this seed, a launch of about 30 s; the full budgets
    total 3.8e9 paths). Creating the batch autotunes
    its launch shape on a sample of its photons, so the one launch timed here is warm."""
    rng = np.random.default_rng(seed)
    insts = []
    ray_cache = None
    for i in range(n_inst):
        if rng.random() < 0.5:
            sc = M.RayleighScatterer(1.0, 1.0)
        else:
            x = rng.uniform(0.5, 10.0)
            m = complex(rng.uniform(1.3, 1.6), 10 ** rng.uniform(-5, -2))
            sc = M.MieScatterer(x / (2 * math.pi), m, 1.0, 0.1, Ntheta=1801)
        tau = 10 ** rng.uniform(-1, math.log10(50))
        omega = rng.uniform(0.5, 0.9999)
        g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=tau * sc.kl, scatterer=sc, omega=omega)])
        n = max(1, int(rng.lognormal(math.log(1e7), 1.0) * scale))
        insts.append({"geometry": g, "I0": [1.0, 0.0, 0.0, 0.0], "n_photons": n, "seed": seed, "instance": i})
        ray_cache = ray_cache or g
    cfg = M.Config(ray_cache, number_of_rays=1)
    b = M.Batch(cfg, insts, ctx=ctx, precision="fp32")
    b.launch()
    ms, photons = b.timing()
    b.close()
    return {"instances": n_inst, "budget_scale": scale, "photons": photons, "kernel_ms": ms,
            "paths_per_s": photons / (ms / 1e3)}


def _scale(b):
    """The largest |I| of a Stokes tally (shape (4, ...)), else the largest |b|."""
    b = np.asarray(b, float)
    return float(np.max(np.abs(b[0]))) if b.ndim >= 2 and b.shape[0] == 4 else float(np.max(np.abs(b)))


def _scaled_err(a, b):
    """max |a - b| over the largest |I| of b (Stokes tallies of shape (4, ...))."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    scale = _scale(b)
    return float(np.max(np.abs(a - b)) / scale) if scale > 0 else float(np.max(np.abs(a)))


ERR_FLOOR = 1e-3  # per-element errors are stated on the elements with |b| >= ERR_FLOOR * scale


def _fp32_err(a, b):
    """FP32-against-FP64 error of one tally: the scaled error, and the per-element relative
    error |a - b| / |b| over the elements above ERR_FLOOR of the tally's scale."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    m = np.abs(b) >= ERR_FLOOR * _scale(b)
    pe = float(np.max(np.abs(a[m] - b[m]) / np.abs(b[m]))) if np.any(m) else 0.0
    return {"scaled": _scaled_err(a, b), "per_element_max": pe, "elements": int(m.sum()), "of": int(b.size)}


def _fp32_errs(r32, r64):
    out = {k: _fp32_err(r32[k], r64[k]) for k in ("A", "Irt", "Icb", "ladder")}
    out["floor"] = ERR_FLOOR
    return out


def other_workloads_leg(M, ctx, n32=1 << 16, n64=None):
    """The Rayleigh slab (Nθ = 180, 200 CB angles over 0-2°, τ = 10, ω = 0.99, normal
    incidence, at most 1000 orders) and the Mie sphere (τ = 20, x = 2, m = 1.31, 500 CB
    angles over 0-5°): FP32 paths/s, FP64 paths/s, and the FP32-vs-FP64 error of every
    tally on identical Philox streams. FP64 runs at about 1/64 of the FP32 rate on this
    GPU, so its samples are 2^14 (slab) and 2^13 (sphere) photons."""
    n64 = n64 or {"rayleigh_slab_tau10": 1 << 14, "mie_sphere_tau20": 1 << 13}
    I0 = [1.0, 0.0, 0.0, 0.0]
    ray = M.RayleighScatterer(0.99, 100.0)
    g1 = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=10 * ray.kl, scatterer=ray)])
    tb1 = [math.radians(2.0) * i / 199 for i in range(200)]
    mie2 = M.MieScatterer(2.0 / (2 * math.pi), 1.31 + 0j, 1.0, 0.1, Ntheta=1801)
    g3 = M.SphereGeometry(R=20 * mie2.kl, scatterer=mie2)
    tb3 = [math.radians(5.0) * i / 499 for i in range(500)]
    runs = (("rayleigh_slab_tau10", g1, lambda n: M.Config(g1, number_of_rays=n, Ntheta=180, thetab=tb1,
                                                             maximum_scattering_times=1000), 1),
            ("mie_sphere_tau20", g3, lambda n: M.Config(g3, number_of_rays=n, thetab=tb3), 3))
    out = {}
    for name, g, mk, seed in runs:
        r32 = M.simulate(mk(n32), g, I0, ctx=ctx, precision="fp32", seed=seed, with_extras=True)
        n = n64[name]
        res = {}
        for prec in ("fp32", "fp64"):
            s = M.Solve(mk(n), g, I0, ctx=ctx, precision=prec, seed=seed + 100)
            s.launch(0, n)
            res[prec] = s.read()
            s.close()
        out[name] = {
            "fp32_paths_per_s": n32 / (r32[7]["stats"]["kernel_ms"] / 1e3), "fp32_photons": n32,
            "fp64_paths_per_s": n / (res["fp64"]["stats"]["kernel_ms"] / 1e3), "fp64_photons": n,
            "events_per_path": r32[7]["stats"]["events"] / n32,
            "fp32_vs_fp64": dict(_fp32_errs(res["fp32"], res["fp64"]), photons=n),
        }
    return out


def oracle_workload(O, n_rays):
    """The same workload built from the oracle's own types (its own bhmie and Config), so
    that the CPU legs never load the library."""
    mie = O.MieScatterer(5.0 / (2 * math.pi), 1.5 + 0.001j, 1.0, 0.1, Ntheta=1801)
    g = O.PlaneGeometry(math.radians(150.0), 0.0, [O.Layer(d=5.0 * mie.kl, scatterer=mie)])
    return mie, g, O.Config(g, number_of_rays=n_rays)


def cpu_oracle_rate(n_sample, threads=0):
    """Times the oracle (the FP64 C++ restatement of the reference's CPU path) on a bounded
    sample of the same workload with all host threads."""
    if os.path.join(ROOT, "oracle") not in sys.path:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    mie, g, cfg = oracle_workload(O, n_sample)
    t0 = time.perf_counter()
    O.simulate(cfg, g, [1.0, 0.0, 0.0, 0.0], seed=11, threads=threads)
    dt = time.perf_counter() - t0
    cores = threads if threads > 0 else (os.cpu_count() or 1)
    return n_sample / dt, cores, dt


def run_reference(args, rank):
    """The reference arm: the reference's CPU algorithm (as the FP64 C++ oracle port,
    since Julia is not installed) on the host's cores, same workload and metric. It
    loads only the oracle: its Mie tables and Config come from the oracle's own
    restatement of the reference."""
    if rank != 0:
        return
    rates = []
    for _ in range(max(args.warmup, 0)):
        cpu_oracle_rate(max(args.cpu_sample // 4, 100))
    for _ in range(args.steps):
        r, cores, dt = cpu_oracle_rate(args.cpu_sample)
        rates.append(r)
    v = float(np.mean(rates))
    line = {
        "impl": "reference", "metric": "photon_paths_per_s", "value": v, "unit": "paths/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "photons_per_step": args.cpu_sample, "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": v, "unit": "paths/s", "cores": cores, "kind": "port",
                         "sample": f"{args.cpu_sample} photons per step of the same workload"},
        "e2e": {"value": v, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "Julia is not installed here, so the reference's CPU path runs as its FP64 C++ "
                "restatement (oracle/mcrt_oracle.cpp) with OpenMP over photons; the Mie tables come "
                "from the oracle's own bhmie, and the library is not loaded",
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if args.impl == "reference":
        run_reference(args, rank)
        if dist:
            dist.destroy_process_group()
        return

    import mcrt_gb300 as M

    if args.case > 0:
        if args.case_workload == "mie_slab":
            mie, g, cfg = workload(M, args.case)
        elif args.case_workload == "rayleigh_slab":
            ray = M.RayleighScatterer(0.99, 100.0)
            g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=10 * ray.kl, scatterer=ray)])
            cfg = M.Config(g, number_of_rays=args.case, Ntheta=180, maximum_scattering_times=1000,
                           thetab=[math.radians(2.0) * i / 199 for i in range(200)])
        else:
            mie2 = M.MieScatterer(2.0 / (2 * math.pi), 1.31 + 0j, 1.0, 0.1, Ntheta=1801)
            g = M.SphereGeometry(R=20 * mie2.kl, scatterer=mie2)
            cfg = M.Config(g, number_of_rays=args.case, thetab=[math.radians(5.0) * i / 499 for i in range(500)])
        out = M.simulate(cfg, g, [1.0, 0.0, 0.0, 0.0], precision=args.case_precision, seed=2,
                         block_size=256, blocks_per_sm=2 if args.case_precision == "fp32" else 1,
                         table_staging="shared", with_extras=True)
        st = out[7]["stats"]
        print(json.dumps({"case_photons": args.case, "kernel_ms": st["kernel_ms"],
                          "paths_per_s": args.case / st["kernel_ms"] * 1e3, "events": st["events"],
                          "rt_evals": st["rt_evals"], "cbn_evals": st["cbn_evals"], "cb1_evals": st["cb1_evals"]}))
        return

    import torch

    ctx = M.Context(local)
    mie, g, cfg = workload(M, args.batch)
    B = args.batch
    I0 = [1.0, 0.0, 0.0, 0.0]
    solve = M.Solve(cfg, g, I0, ctx=ctx, precision="fp32", seed=2)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")  # > L2 (129 MB)

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    step_photons = lambda s: (s * world + rank) * B  # photon_begin of this rank's shard
    for s in range(args.warmup):
        solve.launch(step_photons(s), B)
        solve.read()
    clocks = Clocks(local)
    barrier()
    kms, stats = [], []
    raw = np.zeros(5 + 4 * cfg.Ntheta * cfg.Nphi + 5 * cfg.Nthetab * cfg.Nphib + 1)
    wall0 = time.perf_counter()
    for s in range(args.steps):
        flush.fill_(s & 0xFF)  # evict L2 between timed steps (outside the kernel's events)
        torch.cuda.synchronize()
        solve.launch(step_photons(args.warmup + s), B)
        r = solve.read()
        kms.append(r["stats"]["kernel_ms"])
        stats.append(r["stats"])
        raw += np.concatenate([r["A"], r["Irt"].ravel(), r["Icb"].ravel(), r["ladder"].ravel(),
                               [r["stats"]["photons"]]])
    barrier()
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    t_dev = sum(kms) / 1e3
    if dist:
        t = torch.tensor([t_dev], device=f"cuda:{local}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_dev = float(t.item())
    value = world * B * args.steps / t_dev
    # The sharded form's one exchange: the ranks' raw tallies summed once, after the timed
    # region (a single all-reduce of about 0.1 MB).
    if dist:
        t = torch.from_numpy(raw).to(f"cuda:{local}")
        dist.all_reduce(t)
        raw = t.cpu().numpy()
    n_all = raw[-1]
    tallies = {"ranks_summed": world, "photons": float(n_all), "energy_closure_err": float(abs(raw[:5].sum() / n_all - 1)),
               "cb_peak_s11": float(raw[5 + 4 * cfg.Ntheta * cfg.Nphi] / n_all)}

    # ---- e2e: the drop-in call with host buffers (uploads, launch, copy back, free)
    e2e_times = []
    h2d = d2h = 0
    for s in range(args.steps):
        barrier()
        t0 = time.perf_counter()
        out = M.simulate(cfg, g, I0, ctx=ctx, precision="fp32", seed=3,
                         photon_begin=step_photons(args.warmup + args.steps + s), with_extras=True)
        e2e_times.append(time.perf_counter() - t0)
    nrt, ncb = 4 * cfg.Ntheta * cfg.Nphi, 4 * cfg.Nthetab * cfg.Nphib
    d2h = 8 * (nrt + ncb + ncb // 4 + 16)
    h2d = 8 * (2 * cfg.Ntheta * 4 + 2 * cfg.Nphi + cfg.Nthetab * cfg.Nphib * 12 + 2 * cfg.Nthetab
               + 2 * cfg.Nphib) // 2 + 2048  # FP32 bin tables + the instance descriptor
    e2e_t = sum(e2e_times)
    if dist:
        t = torch.tensor([e2e_t], device=f"cuda:{local}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_t = float(t.item())
    e2e = {"value": world * B * args.steps / e2e_t, "unit": "paths/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "call": "mcrt_simulate (C ABI, host buffers)"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    # ---- CB peak variance -> paths needed for 1% relative standard error
    S = sum(st["cb_peak_sum"] for st in stats)
    SS = sum(st["cb_peak_sumsq"] for st in stats)
    N = sum(st["photons"] for st in stats)
    mu = S / N
    var = max(SS / N - mu * mu, 0.0)
    paths_1pct = var / (0.01 * mu) ** 2 if mu > 0 else float("inf")
    events = sum(st["events"] for st in stats)
    rt = sum(st["rt_evals"] for st in stats)
    cb1 = sum(st["cb1_evals"] for st in stats)
    cbn = sum(st["cbn_evals"] for st in stats)
    flops = rt * FLOPS_RT_MIE + cbn * FLOPS_CBN_MIE + cb1 * FLOPS_CB1_MIE  # this rank's (one GPU's) work
    achieved = flops / t_dev / 1e12
    peak = ctx.fp32_peak_tflops()
    traffic = None
    if NCU_DRAM_BYTES_PER_PHOTON is not None:
        traffic = NCU_DRAM_BYTES_PER_PHOTON * B

    extras = {}
    # The extra legs (FP64 forms, CPU baseline, serving, batches, other workloads) run at
    # N = 1 only: with more ranks the other GPUs would sit idle while rank 0 runs them.
    if not args.no_extras and world == 1:
        # FP64 forms on bounded samples: the same persistent kernel in FP64, and the plain
        # per-ray FP64 kernel with the reference's structure (denominator of the 5x target).
        n64 = args.fp64_sample
        _, g64, cfg64 = workload(M, n64)
        np64 = 4 * n64
        s64 = M.Solve(cfg64.replace(number_of_rays=np64), g64, I0, ctx=ctx, precision="fp64", seed=2)
        s64.launch(0, np64)
        r64 = s64.read()
        s64.close()
        # the FP32 kernel on the same photons and Philox streams: its error against FP64
        s32 = M.Solve(cfg64.replace(number_of_rays=np64), g64, I0, ctx=ctx, precision="fp32", seed=2)
        s32.launch(0, np64)
        r32 = s32.read()
        s32.close()
        err32 = dict(_fp32_errs(r32, r64), photons=np64)
        # The plain per-ray FP64 kernel in two launches, both 256-thread blocks over a
        # grid-stride loop: one thread per photon over the whole GPU (its best measured
        # rate; more photons per thread measured slower: 3.3e3 paths/s at 2 and 3.1e3 at 4
        # on 38 912 threads, against 4.6e3 at 1), and the reference's own launch,
        # threads = min(maximum_threads = 8192, rays) (src/config.jl:69,
        # src/MonteCarloRadiativeTransfer.jl:39,46), which fills 32 of the 152 SMs.
        def plain_rate(threads, photons):
            sp = M.Solve(cfg64.replace(number_of_rays=photons, maximum_threads=threads), g64, I0, ctx=ctx,
                         precision="fp64", kernel="plain", seed=2)
            sp.launch(0, photons)
            rp = sp.read()
            sp.close()
            return photons / (rp["stats"]["kernel_ms"] / 1e3), rp["stats"]["blocks"]

        plain_threads = min(n64, 65536)
        vplain, plain_blocks = plain_rate(plain_threads, n64)
        ref_threads, ref_ppt = 8192, 2
        vplain_ref, ref_blocks = plain_rate(ref_threads, ref_threads * ref_ppt)
        v64 = np64 / (r64["stats"]["kernel_ms"] / 1e3)
        cpu_v, cores, cpu_dt = cpu_oracle_rate(args.cpu_baseline_sample)
        serve = serve_leg(M, ctx, args.serve_requests, args.serve_scale) if args.serve_requests > 0 else None
        batch = batch_leg(M, ctx)
        others = other_workloads_leg(M, ctx)
        # the CB peak's standard error from batch means over 32 photon sub-ranges, beside
        # the per-path estimate on the same photons
        bm = M.cb_peak_batch_means(cfg, g, I0, batches=32, photons_per_batch=1 << 16, ctx=ctx,
                                   precision="fp32", seed=3)
        extras = {
            "other_workloads": others,
            "serve": serve,
            "batch_uneven_slabs": batch,
            "fp64_persistent": {"value": v64, "unit": "paths/s", "sample_photons": np64},
            "fp64_plain": {"value": vplain, "unit": "paths/s", "sample_photons": n64,
                           "threads": plain_threads, "blocks": plain_blocks, "block_size": 256,
                           "photons_per_thread": n64 / plain_threads,
                           "note": "the plain kernel's best measured rate (one photon per thread over the "
                                   "whole GPU) is the denominator of fp32_over_fp64_plain"},
            "fp64_plain_reference_launch": {"value": vplain_ref, "unit": "paths/s",
                                            "sample_photons": ref_threads * ref_ppt, "threads": ref_threads,
                                            "blocks": ref_blocks, "block_size": 256,
                                            "photons_per_thread": ref_ppt},
            "fp32_vs_fp64": err32,
            "fp32_over_fp64_plain": value / world / vplain,
            "fp32_over_fp64_plain_reference_launch": value / world / vplain_ref,
            "fp32_over_fp64_persistent": value / world / v64,
            "cpu_baseline": {"value": cpu_v, "unit": "paths/s", "cores": cores, "kind": "port",
                             "sample": f"{args.cpu_baseline_sample} photons of the same workload, FP64, "
                                       f"{cpu_dt:.1f} s"},
        }

    line = {
        "metric": "photon_paths_per_s", "value": value, "unit": "paths/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "photons_per_step_per_gpu": B,
                   "photons_timed": world * B * args.steps, "full_workload_photons": FULL_WORKLOAD_PHOTONS,
                   "bins": {"Ntheta": cfg.Ntheta, "Nphi": cfg.Nphi, "Ntheta_b": cfg.Nthetab,
                            "Nphi_b": cfg.Nphib},
                   "mie_table_angles": 1801, "parallelism": f"photon shards x{world}",
                   "l2": "flushed between timed steps (256 MB write)",
                   "launch": {"block_size": stats[0]["block_size"], "blocks": stats[0]["blocks"]}},
        "e2e": e2e,
        "gpu_launches": args.steps,
        "tallies": tallies,
        "wall_s_timed": wall,
        "cb_peak": {"mean_per_path": mu, "std_per_path": math.sqrt(var),
                    "paths_for_1pct_stderr": paths_1pct,
                    "seconds_to_1pct_fp32": paths_1pct / value},
        "events_per_path": events / N,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": "live FP32 FFMA microbenchmark (mcrt_measure_fp32_peak)",
                     "flops_per_unit": {"rt_bin": FLOPS_RT_MIE, "cb_reciprocal_bin": FLOPS_CBN_MIE,
                                        "cb_single_bin": FLOPS_CB1_MIE}},
        "clocks": clk,
    }
    line.update(extras)
    if "fp64_plain" in extras:
        line["cb_peak"]["seconds_to_1pct_fp64_plain"] = paths_1pct / extras["fp64_plain"]["value"]
        line["cb_peak"]["batch_means"] = bm
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
