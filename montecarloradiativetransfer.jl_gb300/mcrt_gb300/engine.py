"""simulate / run_rt on the GPU through libmcrt, mirroring the reference's driver
(src/MonteCarloRadiativeTransfer.jl:26-291).
"""
from __future__ import annotations

import ctypes as C
import json
import math
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from ._lib import check, dptr, lib

_PREC = {"fp32": _lib.FP32, "fp64": _lib.FP64}
_KERN = {"persistent": _lib.KERNEL_PERSISTENT, "plain": _lib.KERNEL_PLAIN}


class Context:
    """One CUDA device: the library context plus uploaded scatterers (by identity)."""

    def __init__(self, device: int = 0):
        L = lib()
        if L.mcrt_device_count() <= 0:
            raise _lib.MCRTError(_lib.MCRT_ENODEV, "no CUDA device is visible")
        h = C.c_void_p()
        check(L.mcrt_ctx_create(int(device), C.byref(h)))
        self.h = h
        self.device = device
        self._scat: Dict[int, Tuple[object, C.c_void_p]] = {}
        self._owned: List[C.c_void_p] = []

    def scatterer(self, s) -> C.c_void_p:
        if isinstance(s, DeviceMieScatterer):
            if s.ctx is not self:
                raise ValueError("this scatterer's tables live on another context's device")
            return s.handle
        key = id(s)
        hit = self._scat.get(key)
        if hit is not None and hit[0] is s:
            return hit[1]
        d = _lib.ScattererDesc()
        d.kind, d.omega, d.kl = s.kind, s.omega, s.kl
        keep = []
        if s.kind == _lib.MIE:
            F = [np.ascontiguousarray(a, float) for a in (s.F11, s.F12, s.F33, s.F34)]
            S = [np.ascontiguousarray(np.column_stack([z.real, z.imag]).ravel()) for z in (s.S11, s.S22)]
            cs = np.ascontiguousarray(s.csrn, float)
            keep = F + S + [cs]
            d.n_theta = len(F[0])
            d.F11, d.F12, d.F33, d.F34 = (dptr(a) for a in F)
            d.S11, d.S22 = dptr(S[0]), dptr(S[1])
            d.random_points = len(cs) - 1
            d.csrn = dptr(cs)
        h = C.c_void_p()
        check(lib().mcrt_scatterer_create(self.h, C.byref(d), C.byref(h)))
        del keep
        self._scat[key] = (s, h)
        return h

    def geometry_c(self, g):
        """C view of a geometry; returns (GeometryC, keep-alive list)."""
        if g.kind == _lib.PLANE:
            layers = (_lib.LayerC * len(g.layers))()
            for i, l in enumerate(g.layers):
                layers[i] = _lib.LayerC(l.tau, l.omega, int(l.infinite), self.scatterer(l.scatterer))
            gc = _lib.GeometryC(_lib.PLANE, g.theta, g.phi, len(g.layers), layers)
        else:
            layers = (_lib.LayerC * 1)()
            layers[0] = _lib.LayerC(g.tau, g.omega, 0, self.scatterer(g.scatterer))
            gc = _lib.GeometryC(_lib.SPHERE, math.pi, 0.0, 1, layers)
        return gc, [layers]

    def mie_scatterers(self, params: Sequence[Tuple[float, complex, float, float]], *, Ntheta: int = 181,
                       random_points: int = 1000, with_tables: bool = False) -> List["DeviceMieScatterer"]:
        """MieScatterer(r, m, λ, ν; Nθ, random_points) for each (r, m, λ, ν) in ``params``,
        with bhmie and calculate_csrn run on the device in one launch
        (mcrt_mie_scatterers_create); the tables stay in device memory. With
        ``with_tables`` the FP64 tables are also copied back onto the returned objects."""
        n = len(params)
        r, mre, mim, lam, nu = (np.ascontiguousarray([f(p) for p in params], float) for f in (
            lambda p: p[0], lambda p: complex(p[1]).real, lambda p: complex(p[1]).imag, lambda p: p[2],
            lambda p: p[3]))
        nres = 7 + 8 * Ntheta + random_points + 1
        tab = np.zeros(n * nres) if with_tables else None
        hs = (C.c_void_p * n)()
        check(lib().mcrt_mie_scatterers_create(self.h, n, dptr(r), dptr(mre), dptr(mim), dptr(lam), dptr(nu),
                                               int(Ntheta), int(random_points), hs,
                                               dptr(tab) if tab is not None else None))
        out = []
        for i in range(n):
            h = C.c_void_p(hs[i])
            self._owned.append(h)
            out.append(DeviceMieScatterer(self, h, params[i], Ntheta, random_points,
                                          tab[i * nres:(i + 1) * nres] if tab is not None else None))
        return out

    def fp32_peak_tflops(self) -> float:
        v = np.zeros(1)
        check(lib().mcrt_measure_fp32_peak(self.h, dptr(v)))
        return float(v[0])

    def close(self) -> None:
        if self.h:
            L = lib()
            for _, h in self._scat.values():
                L.mcrt_scatterer_destroy(h)
            self._scat.clear()
            for h in self._owned:
                L.mcrt_scatterer_destroy(h)
            self._owned.clear()
            L.mcrt_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceMieScatterer:
    """A MieScatterer whose tables were produced on, and stay on, one context's device
    (Context.mie_scatterers). It stands wherever a MieScatterer does in a Layer or a
    SphereGeometry run on that context."""

    kind = _lib.MIE

    def __init__(self, ctx: "Context", handle: C.c_void_p, param, Ntheta: int, random_points: int, tables=None):
        self.ctx, self.handle = ctx, handle
        self.r, self.m, self.lam, self.nu = float(param[0]), complex(param[1]), float(param[2]), float(param[3])
        self.x = 2 * math.pi * self.r / self.lam
        self.Ntheta, self.random_points = int(Ntheta), int(random_points)
        om, kl = C.c_double(), C.c_double()
        check(lib().mcrt_scatterer_params(handle, C.byref(om), C.byref(kl)))
        self.omega, self.kl = om.value, kl.value
        if tables is not None:
            n, rp = self.Ntheta, self.random_points
            self.q_ext, self.q_sca, self.q_abs, self.q_back, self.asymm = (float(v) for v in tables[2:7])
            o = 7
            self.F11, self.F12, self.F33, self.F34 = (tables[o + k * n:o + (k + 1) * n].copy() for k in range(4))
            o += 4 * n
            self.S11 = tables[o:o + 2 * n:2] + 1j * tables[o + 1:o + 2 * n:2]
            o += 2 * n
            self.S22 = tables[o:o + 2 * n:2] + 1j * tables[o + 1:o + 2 * n:2]
            o += 2 * n
            self.csrn = tables[o:o + rp + 1].copy()

    def __repr__(self) -> str:
        return f"DeviceMieScatterer(x={self.x:.6g}, m={self.m}, omega={self.omega:.6g}, kl={self.kl:.6g})"


_default: Optional[Context] = None


def default_context() -> Context:
    global _default
    if _default is None:
        _default = Context(0)
    return _default


_STAGING = {"auto": 0, "shared": 1, "global": 2}


def run_opts(precision="fp32", kernel="persistent", seed=1, instance=0, rng_mode=0, photon_begin=0,
             block_size=0, blocks_per_sm=0, plain_threads=0, table_staging="auto",
             max_attempts=0) -> _lib.RunOpts:
    """Launch options (mcrt_run_opts). Zero block_size / blocks_per_sm and "auto" staging
    leave the choice to the library's autotuner; zero max_attempts keeps the default
    rejection-loop cap (2^20)."""
    return _lib.RunOpts(_PREC[precision], _KERN[kernel], int(seed), int(instance), int(rng_mode),
                        int(photon_begin), int(block_size), int(blocks_per_sm), int(plain_threads),
                        _STAGING[table_staging], int(max_attempts))


def _views(cfg, Irt, Icb, lad):
    """Reference layouts: Irt[s, j1, j2] of shape (4, Ntheta, Nphi), Icb (4, Ntheta_b, Nphi_b)."""
    irt = Irt.reshape(cfg.Nphi, cfg.Ntheta, 4).transpose(2, 1, 0)
    icb = Icb.reshape(cfg.Nphib, cfg.Nthetab, 4).transpose(2, 1, 0)
    ld = lad.reshape(cfg.Nphib, cfg.Nthetab).T
    return irt, icb, ld


def simulate(cfg, g, I0, *, use_gpu: bool = True, ctx: Optional[Context] = None, with_extras: bool = False,
             **opts):
    """simulate(cfg, g, I0; use_gpu) of src/MonteCarloRadiativeTransfer.jl:26-85.

    Returns ``(Adt, Aabs, Aref, Atrans, Arem, Irt, Icb)`` divided by ``number_of_rays``,
    with ``Irt`` of shape (4, Ntheta, Nphi) and ``Icb`` of shape (4, Ntheta_b, Nphi_b).
    ``opts`` are the launch options of :func:`run_opts` (precision, kernel, seed,
    instance, rng_mode, ...). With ``with_extras`` an eighth element is a dict holding
    the incoherent CB tally ``ladder`` and the launch ``stats``.
    """
    if not use_gpu:
        raise NotImplementedError(
            "this package runs the transport on the GPU only; the CPU path is the reference's")
    ctx = ctx or default_context()
    g.validate()
    cc = cfg.to_c()
    gc, keep = ctx.geometry_c(g)
    I = np.ascontiguousarray(I0, float)
    A = np.zeros(5)
    Irt = np.zeros(4 * cfg.Ntheta * cfg.Nphi)
    Icb = np.zeros(4 * cfg.Nthetab * cfg.Nphib)
    lad = np.zeros(cfg.Nthetab * cfg.Nphib)
    st = _lib.Stats()
    o = run_opts(**opts)
    check(lib().mcrt_simulate(ctx.h, C.byref(cc), C.byref(gc), dptr(I), C.byref(o), dptr(A),
                              dptr(Irt), dptr(Icb), dptr(lad), C.byref(st)))
    irt, icb, ld = _views(cfg, Irt, Icb, lad)
    out = (A[0], A[1], A[2], A[3], A[4], irt, icb)
    if with_extras:
        return out + ({"ladder": ld, "stats": st.as_dict()},)
    return out


class Solve:
    """A resident solve: inputs and tallies stay on the device between launches."""

    def __init__(self, cfg, g, I0, *, ctx: Optional[Context] = None, **opts):
        self.ctx = ctx or default_context()
        g.validate()
        self.cfg = cfg
        self._cc = cfg.to_c()
        self._gc, self._keep = self.ctx.geometry_c(g)
        self._I = np.ascontiguousarray(I0, float)
        self._o = run_opts(**opts)
        h = C.c_void_p()
        check(lib().mcrt_solve_create(self.ctx.h, C.byref(self._cc), C.byref(self._gc), dptr(self._I),
                                      C.byref(self._o), C.byref(h)))
        self.h = h
        n = cfg
        self.A = np.zeros(5)
        self.Irt = np.zeros(4 * n.Ntheta * n.Nphi)
        self.Icb = np.zeros(4 * n.Nthetab * n.Nphib)
        self.lad = np.zeros(n.Nthetab * n.Nphib)
        self.stats = _lib.Stats()

    def launch(self, photon_begin: int, n_photons: int) -> None:
        check(lib().mcrt_solve_launch(self.h, int(photon_begin), int(n_photons)))

    def read(self) -> dict:
        """Raw (undivided) sums of the last launch."""
        check(lib().mcrt_solve_read(self.h, dptr(self.A), dptr(self.Irt), dptr(self.Icb), dptr(self.lad),
                                    C.byref(self.stats)))
        irt, icb, ld = _views(self.cfg, self.Irt, self.Icb, self.lad)
        return {"A": self.A.copy(), "Irt": irt.copy(), "Icb": icb.copy(), "ladder": ld.copy(),
                "stats": self.stats.as_dict()}

    def close(self) -> None:
        if self.h:
            lib().mcrt_solve_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def simulate_to_stderr(cfg, g, I0, rel_err: float = 0.01, *, batch: int = 1 << 20, max_photons: int = 1 << 34,
                       ctx: Optional[Context] = None, state: Optional[dict] = None, **opts):
    """simulate() until the CB peak (s11 of Icb at θb = 0) is known to ``rel_err``.

    Launches of ``batch`` photons run on consecutive photon ranges of one Philox stream
    (so the result equals one simulate() of the same total) until the standard error of
    the per-path CB peak, from its per-path sums of x and x², falls to ``rel_err`` of its
    mean, or ``max_photons`` have run. Returns ``(result, info)``: ``result`` is
    simulate()'s tuple for all photons run, ``info`` holds ``photons``, ``rel_err``,
    ``launches`` and ``state``.

    ``state`` is a checkpoint: the raw sums and the photon count so far (plain numpy
    values, e.g. for ``numpy.savez``). Passing it back continues the same stream at the
    next photon, so a stopped run resumes where it left off."""
    if rel_err <= 0:
        raise ValueError("rel_err must be positive")
    s = Solve(cfg.replace(number_of_rays=batch), g, I0, ctx=ctx, **opts)
    try:
        A = Irt = Icb = lad = None
        n = 0
        x = x2 = 0.0
        if state is not None:
            A, Irt, Icb, lad = (np.array(state[k], float) for k in ("A", "Irt", "Icb", "ladder"))
            n, x, x2 = int(state["photons"]), float(state["peak_sum"]), float(state["peak_sumsq"])
        launches = 0
        err = math.inf
        while True:
            s.launch(n, batch)
            r = s.read()
            launches += 1
            n += batch
            if A is None:
                A, Irt, Icb, lad = r["A"], r["Irt"], r["Icb"], r["ladder"]
            else:
                A, Irt, Icb, lad = A + r["A"], Irt + r["Irt"], Icb + r["Icb"], lad + r["ladder"]
            x += r["stats"]["cb_peak_sum"]
            x2 += r["stats"]["cb_peak_sumsq"]
            mean = x / n
            var = max(x2 / n - mean * mean, 0.0)
            err = math.sqrt(var / n) / mean if mean > 0 else math.inf
            if err <= rel_err or n + batch > max_photons:
                break
    finally:
        s.close()
    out = (A[0] / n, A[1] / n, A[2] / n, A[3] / n, A[4] / n, Irt / n, Icb / n)
    ckpt = {"A": A, "Irt": Irt, "Icb": Icb, "ladder": lad, "photons": n, "peak_sum": x, "peak_sumsq": x2}
    return out, {"photons": n, "rel_err": err, "launches": launches, "ladder": lad / n, "state": ckpt}


def peak_error_estimates(sums, sumsqs, n_per_batch: int):
    """Two standard errors of the mean CB peak per path, from ``B`` batches of
    ``n_per_batch`` paths each, given each batch's sums of x and x² over its paths.

    Batch means: the spread of the ``B`` batch averages, ``std(m_b, ddof=1)/sqrt(B)``.
    Per path: ``sqrt((Σx²/N − mean²)/N)`` from the pooled sums. For independent paths
    both estimate the same quantity; their ratio follows ``sqrt(χ²_{B−1}/(B−1))``.
    Returns ``(mean, se_batch_means, se_per_path)``."""
    s = np.asarray(sums, float)
    ss = np.asarray(sumsqs, float)
    if s.ndim != 1 or s.shape != ss.shape or s.size < 2 or n_per_batch < 1:
        raise ValueError("need at least two batches of equal, positive size")
    n_total = s.size * n_per_batch
    mean = float(s.sum()) / n_total
    se_bm = float(np.std(s / n_per_batch, ddof=1)) / math.sqrt(s.size)
    var = max(float(ss.sum()) / n_total - mean * mean, 0.0)
    return mean, se_bm, math.sqrt(var / n_total)


def cb_peak_batch_means(cfg, g, I0, *, batches: int = 32, photons_per_batch: int = 1 << 16,
                        ctx: Optional[Context] = None, **opts) -> dict:
    """The CB peak's standard error from batch means over ``batches`` independent photon
    sub-ranges (consecutive ranges of one Philox stream), beside the per-path estimate
    from the same photons' sums of x and x². Returns a dict with the mean per path, both
    relative errors, and the paths each implies for a 1% relative standard error."""
    if batches < 2:
        raise ValueError("batch means need at least two batches")
    s = Solve(cfg.replace(number_of_rays=photons_per_batch), g, I0, ctx=ctx, **opts)
    sums, sqs = [], []
    try:
        for b in range(batches):
            s.launch(b * photons_per_batch, photons_per_batch)
            st = s.read()["stats"]
            sums.append(st["cb_peak_sum"])
            sqs.append(st["cb_peak_sumsq"])
    finally:
        s.close()
    mean, se_bm, se_pp = peak_error_estimates(sums, sqs, photons_per_batch)
    n = batches * photons_per_batch
    out = {"batches": batches, "photons_per_batch": photons_per_batch, "mean_per_path": mean}
    for name, se in (("batch_means", se_bm), ("per_path", se_pp)):
        rel = se / mean if mean > 0 else math.inf
        out["rel_err_" + name] = rel
        out["paths_for_1pct_" + name] = n * (rel / 0.01) ** 2
    return out


class Batch:
    """Many simulate() instances in one persistent launch (per-instance work queues).

    ``instances`` is a list of dicts with keys geometry, I0, n_photons, seed, instance.
    """

    def __init__(self, cfg, instances: Sequence[dict], *, ctx: Optional[Context] = None, **opts):
        self.ctx = ctx or default_context()
        self.cfg = cfg
        self._cc = cfg.to_c()
        n = len(instances)
        self._keep = []
        arr = (_lib.InstanceC * n)()
        self._gcs = []
        for i, d in enumerate(instances):
            d["geometry"].validate()
            gc, keep = self.ctx.geometry_c(d["geometry"])
            self._gcs.append(gc)
            self._keep.append(keep)
            arr[i].geometry = C.pointer(gc)
            for s in range(4):
                arr[i].I0[s] = float(d["I0"][s])
            arr[i].seed = int(d.get("seed", 1))
            arr[i].instance = int(d.get("instance", i))
            arr[i].n_photons = int(d["n_photons"])
        self._arr = arr
        self._o = run_opts(**opts)
        h = C.c_void_p()
        check(lib().mcrt_batch_create(self.ctx.h, C.byref(self._cc), arr, n, C.byref(self._o), C.byref(h)))
        self.h = h
        self.n = n

    def launch(self) -> None:
        check(lib().mcrt_batch_launch(self.h))

    def read(self, i: int) -> dict:
        cfg = self.cfg
        A = np.zeros(5)
        Irt = np.zeros(4 * cfg.Ntheta * cfg.Nphi)
        Icb = np.zeros(4 * cfg.Nthetab * cfg.Nphib)
        lad = np.zeros(cfg.Nthetab * cfg.Nphib)
        st = _lib.Stats()
        check(lib().mcrt_batch_read(self.h, int(i), dptr(A), dptr(Irt), dptr(Icb), dptr(lad), C.byref(st)))
        irt, icb, ld = _views(cfg, Irt, Icb, lad)
        return {"A": A, "Irt": irt, "Icb": icb, "ladder": ld, "stats": st.as_dict()}

    def timing(self) -> Tuple[float, float]:
        ms = np.zeros(1)
        ph = np.zeros(1)
        check(lib().mcrt_batch_timing(self.h, dptr(ms), dptr(ph)))
        return float(ms[0]), float(ph[0])

    def close(self) -> None:
        if self.h:
            lib().mcrt_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """The continuous-batching request loop of libmcrt (mcrt_server_*).

    ``submit`` queues a simulate() request and returns a ticket; ``result`` waits for it
    and returns ``(A, Irt, Icb, ladder, info)`` divided by the request's photon count,
    where ``info`` holds the submit / admit / completion times and the waves it took.
    With ``log_path`` every result also appends one JSON line (ticket, photons, latency,
    queueing time, waves) to that file."""

    def __init__(self, *, ctx: Optional[Context] = None, memory_cap_bytes: float = 20e9, max_active: int = 256,
                 wave_photons: int = 1 << 20, min_quantum: int = 4096, precision: str = "fp32",
                 use_graphs: bool = True, log_path: Optional[str] = None, wave_work: float = 0.0):
        self.ctx = ctx or default_context()
        self._log = open(log_path, "a", encoding="utf-8") if log_path else None
        o = _lib.ServerOpts(float(memory_cap_bytes), int(max_active), int(wave_photons), int(min_quantum),
                            _PREC[precision], int(use_graphs), float(wave_work))
        h = C.c_void_p()
        check(lib().mcrt_server_create(self.ctx.h, C.byref(o), C.byref(h)))
        self.h = h
        self._shapes = {}

    def submit(self, cfg, g, I0, n_photons: int, seed: int = 1, instance: int = 0) -> int:
        g.validate()
        cc = cfg.to_c()
        gc, keep = self.ctx.geometry_c(g)
        r = _lib.RequestC(C.pointer(cc), C.pointer(gc), (C.c_double * 4)(*[float(v) for v in I0]), int(seed),
                          int(instance), int(n_photons))
        t = C.c_uint64()
        check(lib().mcrt_server_submit(self.h, C.byref(r), C.byref(t)))  # the server copies the request
        self._shapes[t.value] = (cfg.Ntheta, cfg.Nphi, cfg.Nthetab, cfg.Nphib)
        return t.value

    def wait(self, ticket: int, timeout_ms: float = 1e9) -> bool:
        rc = lib().mcrt_server_wait(self.h, int(ticket), float(timeout_ms))
        if rc == _lib.MCRT_ETIMEDOUT:
            return False
        check(rc)
        return True

    def result(self, ticket: int, timeout_ms: float = 1e9):
        if not self.wait(ticket, timeout_ms):
            raise TimeoutError(f"ticket {ticket} not done within {timeout_ms} ms")
        nt, nph, ntb, npb = self._shapes.pop(ticket)
        A = np.zeros(5)
        Irt = np.zeros(4 * nt * nph)
        Icb = np.zeros(4 * ntb * npb)
        lad = np.zeros(ntb * npb)
        info = _lib.TicketInfo()
        check(lib().mcrt_server_result(self.h, int(ticket), dptr(A), dptr(Irt), dptr(Icb), dptr(lad),
                                       C.byref(info)))
        irt = Irt.reshape(nph, nt, 4).transpose(2, 1, 0)
        icb = Icb.reshape(npb, ntb, 4).transpose(2, 1, 0)
        d = info.as_dict()
        if self._log:
            self._log.write(json.dumps({"ticket": int(ticket), "photons": d["photons"], "waves": d["waves"],
                                        "latency_s": d["completed_s"] - d["submitted_s"],
                                        "queued_s": d["admitted_s"] - d["submitted_s"]}) + "\n")
            self._log.flush()
        return A, irt, icb, lad.reshape(npb, ntb).T, d

    def stats(self) -> dict:
        v = np.zeros(8)
        check(lib().mcrt_server_stats(self.h, dptr(v)))
        keys = ["completed", "photons", "waves", "busy_s", "peak_resident_bytes", "resident_bytes", "pending",
                "active"]
        return dict(zip(keys, v.tolist()))

    def close(self) -> None:
        if self.h:
            lib().mcrt_server_destroy(self.h)
            self.h = None
        if self._log:
            self._log.close()
            self._log = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------ run_rt
def run_rt(cfg, g, *, use_gpu: bool = True, ctx: Optional[Context] = None, with_stats: bool = False, **opts):
    """run_rt (src/MonteCarloRadiativeTransfer.jl:87-291): the Mueller matrices of the
    reflected (RT) and coherently backscattered (CB) light, as dicts of columns
    ``theta`` (and ``phi`` for a plane), ``s11`` ... ``s44``, plus an ``energy`` dict.

    All incident polarisation states run in one batched launch of the persistent kernel
    (state i with Philox ``instance + i``) and a device epilogue assembles the matrices
    (mcrt_run_rt). With ``with_stats`` a fourth element holds the summed launch stats."""
    if not use_gpu:
        raise NotImplementedError(
            "this package runs the transport on the GPU only; the CPU path is the reference's")
    ctx = ctx or default_context()
    g.validate()
    cc = cfg.to_c()
    gc, keep = ctx.geometry_c(g)
    plane = g.kind != _lib.SPHERE
    nrt = 16 * cfg.Ntheta * (cfg.Nphi if plane else 1)
    ncb = 16 * cfg.Nthetab * (cfg.Nphib if plane else 1)
    Mrt, Mcb, E = np.zeros(nrt), np.zeros(ncb), np.zeros(5)
    st = _lib.Stats()
    o = run_opts(**opts)
    check(lib().mcrt_run_rt(ctx.h, C.byref(cc), C.byref(gc), C.byref(o), dptr(Mrt), dptr(Mcb), dptr(E),
                            C.byref(st)))
    Mrt = Mrt.reshape(16, -1)
    Mcb = Mcb.reshape(16, -1)
    th = 180.0 / math.pi * np.arccos(cfg.costheta)
    thb = 180.0 / math.pi * np.arccos(cfg.costhetab)
    if plane:
        sm_rt = {"theta": np.tile(th, cfg.Nphi), "phi": np.repeat(180.0 / math.pi * cfg.phi, cfg.Ntheta)}
        sm_cb = {"theta": np.tile(thb, cfg.Nphib), "phi": np.repeat(180.0 / math.pi * cfg.phib, cfg.Nthetab)}
        energy = {"direct_transmission": E[0], "absorption": E[1], "reflection": E[2], "transmission": E[3],
                  "remaining": E[4]}
    else:
        sm_rt, sm_cb = {"theta": th}, {"theta": thb}
        energy = {"direct_transmission": E[0], "absorption": E[1], "reflection": E[2], "remaining": E[4]}
    for a in range(4):
        for b in range(4):
            sm_rt[f"s{a + 1}{b + 1}"] = Mrt[4 * a + b].copy()
            sm_cb[f"s{a + 1}{b + 1}"] = Mcb[4 * a + b].copy()
    if with_stats:
        return sm_rt, sm_cb, energy, st.as_dict()
    return sm_rt, sm_cb, energy


def _table_columns(table: dict):
    """The reference's DataFrame columns of a run_rt table, in order: ``θ`` (and ``ϕ`` for
    a plane), then ``s11 .. s44`` (src/MonteCarloRadiativeTransfer.jl:176-182, 280-290).
    Returns ``[(header, float64 array)]``."""
    keys = [k for k in ("theta", "phi") if k in table] + [f"s{a}{b}" for a in range(1, 5) for b in range(1, 5)]
    names = {"theta": "θ", "phi": "ϕ"}
    return [(names.get(k, k), np.asarray(table[k], float)) for k in keys]


def write_csv(table: dict, path: str) -> None:
    """Writes a run_rt table as CSV with the reference's DataFrame headers ``θ, ϕ, s11 .. s44``."""
    cols = _table_columns(table)
    data = np.column_stack([v for _, v in cols])
    with open(path, "w", encoding="utf-8") as f:
        f.write(",".join(h for h, _ in cols) + "\n")
        for row in data:
            f.write(",".join(repr(float(v)) for v in row) + "\n")


def write_arrow(table: dict, path: str) -> None:
    """Writes a run_rt table as an Arrow IPC file (readable as a DataFrame by Arrow.jl or
    pandas) with the reference's column names ``θ, ϕ, s11 .. s44``, all Float64. Needs
    pyarrow, which is imported only here."""
    try:
        import pyarrow as pa
        import pyarrow.ipc as ipc
    except ImportError as e:  # the CSV writer needs nothing
        raise ImportError("write_arrow needs pyarrow; write_csv writes the same table without it") from e
    cols = _table_columns(table)
    t = pa.table({h: pa.array(v, type=pa.float64()) for h, v in cols})
    with pa.OSFile(path, "wb") as sink, ipc.new_file(sink, t.schema) as w:
        w.write_table(t)
