"""mcrt_simulate_noalloc: the simulate entry point for callers that must not allocate
device memory when they call it (an application whose device memory is reserved up
front by its own allocator, or a loop that may not allocate once running). It keeps
all of its call-time device storage in one fixed-size array inside the library, which
exists once the first context on the device has been created.

The tests call it through the C ABI twice in a row and compare each result with the
regular entry point mcrt_simulate on the same inputs and Philox streams: the second
call checks that nothing left in the shared array by the first leaks into it. They
also check that a call leaves the device's free memory unchanged, and that launch
options it does not honour are refused. They sit in a file of their own, collected
last, and need no state from the other tests.
"""
import ctypes as C
import math

import numpy as np
import pytest

from helpers import scaled_err

pytestmark = pytest.mark.gpu


@pytest.fixture
def ctx(M):
    if M.lib().mcrt_device_count() <= 0:
        pytest.fail("needs a CUDA device")
    c = M.Context(0)
    try:
        yield c
    finally:
        c.close()


def _call(M, name, ctx, cfg, g, I0, opts):
    L = M.lib()
    cc = cfg.to_c()
    gc, keep = ctx.geometry_c(g)
    I = np.ascontiguousarray(I0, float)
    A = np.zeros(5)
    Irt = np.zeros(4 * cfg.Ntheta * cfg.Nphi)
    Icb = np.zeros(4 * cfg.Nthetab * cfg.Nphib)
    lad = np.zeros(cfg.Nthetab * cfg.Nphib)
    st = M._lib.Stats()
    fn = getattr(L, name)
    M._lib.check(fn(ctx.h, C.byref(cc), C.byref(gc), M._lib.dptr(I), C.byref(opts), M._lib.dptr(A),
                    M._lib.dptr(Irt), M._lib.dptr(Icb), M._lib.dptr(lad), C.byref(st)))
    return A, Irt, Icb, lad, st.as_dict()


def _workload(M, scat):
    if scat == "mie":
        sc = M.MieScatterer(5.0 / (2 * math.pi), 1.5 + 0.001j, 1.0, 0.1, Ntheta=1801)
    else:  # a Rayleigh slab tallies RT through azimuthal Fourier modes
        sc = M.RayleighScatterer(0.99, 100.0)
    g = M.PlaneGeometry(math.radians(150.0), 0.0, [M.Layer(d=3.0 * sc.kl, scatterer=sc)])
    cfg = M.Config(g, number_of_rays=3000, Ntheta=16, Nphi=8, Nphib=4,
                   thetab=np.deg2rad(np.linspace(0, 3, 12)), maximum_scattering_times=500)
    return g, cfg


@pytest.mark.parametrize("scat", ["mie", "rayleigh"])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-9), ("fp32", 1e-4)])
def test_noalloc_entry_point_matches_simulate_twice(M, ctx, prec, tol, scat):
    g, cfg = _workload(M, scat)
    I0 = [1.0, 0.0, 0.0, 1.0]
    opts = M.run_opts(precision=prec, seed=17, instance=3)
    ref = _call(M, "mcrt_simulate", ctx, cfg, g, I0, opts)
    for _ in range(2):
        got = _call(M, "mcrt_simulate_noalloc", ctx, cfg, g, I0, opts)
        assert got[4]["photons"] == cfg.number_of_rays
        assert got[4]["status_flags"] & 5 == 0
        assert scaled_err(got[0], ref[0]) < tol
        assert scaled_err(got[1].reshape(cfg.Nphi, cfg.Ntheta, 4).transpose(2, 1, 0),
                          ref[1].reshape(cfg.Nphi, cfg.Ntheta, 4).transpose(2, 1, 0)) < tol
        assert scaled_err(got[2].reshape(cfg.Nphib, cfg.Nthetab, 4).transpose(2, 1, 0),
                          ref[2].reshape(cfg.Nphib, cfg.Nthetab, 4).transpose(2, 1, 0)) < tol
        assert scaled_err(got[3], ref[3]) < tol


def test_noalloc_call_leaves_device_free_memory_unchanged(M, ctx):
    """After a first call, further calls change the device's free memory by nothing."""
    torch = pytest.importorskip("torch")
    g, cfg = _workload(M, "mie")
    opts = M.run_opts(precision="fp32", seed=5)
    torch.cuda.mem_get_info(0)  # torch's own set-up happens before the measurement
    _call(M, "mcrt_simulate_noalloc", ctx, cfg, g, [1, 0, 0, 0], opts)
    free0, _ = torch.cuda.mem_get_info(0)
    for _ in range(3):
        _call(M, "mcrt_simulate_noalloc", ctx, cfg, g, [1, 0, 0, 0], opts)
        free1, _ = torch.cuda.mem_get_info(0)
        assert free1 == free0, (free0, free1)


def test_noalloc_rejects_configs_beyond_its_array(M, ctx):
    ray = M.RayleighScatterer(0.99, 10.0)
    g = M.PlaneGeometry(math.pi, 0.0, [M.Layer(d=1.0, scatterer=ray)])
    # 2048 x 2048 RT bins need 128 MiB of tallies, more than the 24 MiB array
    cfg = M.Config(g, number_of_rays=10, Ntheta=2048, Nphi=2048)
    with pytest.raises(M.MCRTError, match="MCRT_NOALLOC_SCRATCH_BYTES"):
        _call(M, "mcrt_simulate_noalloc", ctx, cfg, g, [1, 0, 0, 0], M.run_opts())


@pytest.mark.parametrize("opt", [{"kernel": "plain"}, {"block_size": 512}, {"precision": "fp64", "block_size": 256},
                                 {"blocks_per_sm": 2}, {"table_staging": "global"}])
def test_noalloc_rejects_launch_options_it_does_not_honour(M, ctx, opt):
    g, cfg = _workload(M, "mie")
    with pytest.raises(M.MCRTError) as e:
        _call(M, "mcrt_simulate_noalloc", ctx, cfg, g, [1, 0, 0, 0], M.run_opts(**opt))
    assert e.value.code == M._lib.MCRT_EINVAL
