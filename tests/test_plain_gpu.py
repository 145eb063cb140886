"""Parity of the plain sweep (C ABI, CUDA) with the reference.

Small cases compare against the golden vectors the reference produced
(tests/golden/) and against the CPU oracle run live; the full-size cases
check size-independent properties.

Tolerances (relative max-norm, max|a-b| / max|b|):
  f64   : 1e-12  (the reference's FP64 arithmetic up to FMA contraction and
                  precomputed coefficients)
  f32x2 : 1e-12  (compensated FP32 pairs, ~48 significant bits)
  f32   : 2e-5   (plain FP32; reported, not an FP64-accuracy claim)
"""
from __future__ import annotations

import numpy as np
import pytest

import cases
import oracle as O

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-12, "f32x2": 1e-12, "f32": 2e-5}
PRECS = ["f64", "f32x2", "f32"]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("name", ["heat_noise_16", "heat_noise_odd"])
def test_heat_noise_golden(gpu, name, prec):
    d, cfg, fields = cases.heat_noise(name, prec)
    u = cases.run(cfg, fields, int(d["nsteps"]))
    assert cases.rel_err(u, d["final"]) <= TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_heat_timelin_golden(gpu, prec):
    d, cfg, fields = cases.heat_timelin(prec)
    M = gpu
    T = int(d["nsteps"])
    with M.Plain(cfg) as p:
        for f, a in fields.items():
            p.upload(f, a)
        p.step(T)
        u = p.download()
        err, mx = p.err_linf()
    assert cases.rel_err(u, d["final"]) <= TOL[prec]
    # compErrLinf against the exact solution (1+t)(1+sum x): round-off only.
    assert err / mx <= 10 * TOL[prec]
    assert mx == pytest.approx(float(np.max(np.abs(d["final"]))), rel=1e-12)


@pytest.mark.parametrize("prec", PRECS)
def test_pennes_timelin_golden(gpu, prec):
    d, cfg, fields = cases.pennes_timelin(prec)
    u = cases.run(cfg, fields, int(d["nsteps"]))
    assert cases.rel_err(u, d["final"]) <= TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_stencil_width_one_golden(gpu, prec):
    d, cfg, fields = cases.stencil_width_one(prec)
    u = cases.run(cfg, fields, int(d["nsteps"]))
    assert cases.rel_err(u, d["final"]) <= TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
def test_pennes_mri_golden(gpu, prec):
    d, cfg, fields = cases.pennes_mri(prec)
    u = cases.run(cfg, fields, int(d["nsteps"]))
    assert cases.rel_err(u, d["final"]) <= TOL[prec]


@pytest.mark.parametrize("n", [(3, 3, 3), (4, 3, 5), (33, 7, 65), (5, 40, 9), (64, 17, 3), (31, 33, 35)])
def test_ragged_shapes_vs_oracle(gpu, n):
    M = gpu
    rng = np.random.default_rng(sum(n))
    shape = (n[2], n[1], n[0])
    h2 = sum((m - 1) ** 2 for m in n)
    tau = 0.9 / (2.0 * h2)
    g = O.make_grid(n, tau=tau)
    u0 = rng.uniform(-1.0, 1.0, shape)
    gA = rng.uniform(-1.0, 1.0, shape)
    fA = rng.uniform(-1.0, 1.0, shape)
    T = 17
    ref = O.heat_dirichlet(g, u0, T, coeff_a=1.0, rho_c=2.0, f_base=fA, g_base=gA)
    for prec in PRECS:
        cfg = M.make_cfg(n, tau=tau, precision=prec, heat=(1.0, 2.0, 0.0))
        u = cases.run(cfg, {M.FIELD_F_A: fA, M.FIELD_G_A: gA, M.FIELD_U: u0}, T)
        assert cases.rel_err(u, ref) <= TOL[prec], prec


@pytest.mark.parametrize("n", [(1 << 20, 3, 3), (3, 65536, 3), (5, 3, 1 << 17), (1000, 999, 3)])
def test_extreme_shapes_vs_oracle(gpu, n):
    """Axis extents at the large end of what a handle takes (x up to 2^20
    nodes, long y and z axes, a thin slab): TMA boxes, tile counts and
    z-chunks at their extremes, against the oracle."""
    M = gpu
    rng = np.random.default_rng(7)
    shape = (n[2], n[1], n[0])
    tau = 0.9 / (2.0 * sum((m - 1) ** 2 for m in n))
    g = O.make_grid(n, tau=tau)
    u0 = rng.uniform(-1.0, 1.0, shape)
    gA = rng.uniform(-1.0, 1.0, shape)
    T = 3
    ref = O.heat_dirichlet(g, u0, T, g_base=gA)
    for prec in PRECS:
        cfg = M.make_cfg(n, tau=tau, precision=prec, heat=(1.0, 1.0, 0.0))
        u = cases.run(cfg, {M.FIELD_G_A: gA, M.FIELD_U: u0}, T)
        assert cases.rel_err(u, ref) <= TOL[prec], prec


@pytest.mark.parametrize("tile", [1, 2, 3, 4])
@pytest.mark.parametrize("prec", PRECS)
def test_every_tile_variant(gpu, tile, prec):
    """Each CTA tile variant (32xBY, R rows per thread) on ragged shapes,
    including rows that end inside a thread's row block."""
    M = gpu
    for name in ("heat_noise_odd", "heat_noise_16"):
        d, cfg, fields = cases.heat_noise(name, prec)
        cfg.tile = tile
        u = cases.run(cfg, fields, int(d["nsteps"]))
        assert cases.rel_err(u, d["final"]) <= TOL[prec], name
    d, cfg, fields = cases.stencil_width_one(prec)
    cfg.tile = tile
    u = cases.run(cfg, fields, int(d["nsteps"]))
    assert cases.rel_err(u, d["final"]) <= TOL[prec]


def test_autotune_restores_state(gpu):
    M = gpu
    d, cfg, fields = cases.heat_noise("heat_noise_16", "f64")
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_U, fields[M.FIELD_U])
        p.step(10)
        chosen, ms = p.autotune(5)
        assert 1 <= chosen <= 4 and all(m > 0 for m in ms)
        assert p.timestep() == 10
        p.step(int(d["nsteps"]) - 10)
        u = p.download()
    assert cases.rel_err(u, d["final"]) <= 1e-12


def test_config1_heat_64_full_size_vs_oracle(gpu):
    """64^3, 200 steps, u0 = sin sin sin, tau = 0.9 h^2/6: against the oracle
    and against the analytic decay exp(-3 pi^2 t) u0 (discretisation error)."""
    M = gpu
    n, T = (64, 64, 64), 200
    h = 1.0 / 63
    tau = 0.9 * h * h / 6.0
    g = O.make_grid(n, tau=tau)
    x, y, z = O.coords(g)
    u0 = np.broadcast_to(np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z), (64, 64, 64)).copy()
    u0[O.border_mask(g)] = 0.0
    ref = O.heat_dirichlet(g, u0, T)
    exact = np.exp(-3.0 * np.pi ** 2 * tau * T) * u0
    for prec in ("f64", "f32x2"):
        cfg = M.make_cfg(n, tau=tau, precision=prec, heat=(1.0, 1.0, 0.0))
        u = cases.run(cfg, {M.FIELD_U: u0}, T)
        assert cases.rel_err(u, ref) <= 1e-12, prec
        assert cases.rel_err(u, exact) <= 2e-4, prec


def test_step_counter_and_restart(gpu):
    M = gpu
    d, cfg, fields = cases.heat_noise("heat_noise_16", "f64")
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_U, fields[M.FIELD_U])
        p.step(20)
        p.step(30)
        assert p.timestep() == 50
        a = p.download()
        p.upload(M.FIELD_U, fields[M.FIELD_U])
        assert p.timestep() == 0
        p.step(50)
        b = p.download()
    assert np.array_equal(a, b)
    assert np.array_equal(a, d["final"]) or cases.rel_err(a, d["final"]) <= 1e-12


def test_state_errors(gpu):
    M = gpu
    cfg = M.make_cfg((8, 8, 8), tau=1e-3, heat=(1.0, 1.0, 0.0))
    with M.Plain(cfg) as p:
        with pytest.raises(M.ScafesError) as e:
            p.step(1)
        assert e.value.code == -3
        with pytest.raises(M.ScafesError) as e:
            p.download()
        assert e.value.code == -3
        with pytest.raises(ValueError):
            p.upload(M.FIELD_U, np.zeros(10))
        import ctypes as C
        bad = np.zeros(10)
        rc = M.lib().scafes_gpu_upload(p.h, M.FIELD_U, bad.ctypes.data_as(C.POINTER(C.c_double)), 10)
        assert rc == -1
        rc = M.lib().scafes_gpu_upload(p.h, 99, bad.ctypes.data_as(C.POINTER(C.c_double)), 512)
        assert rc == -1


def test_host_alloc_buffers_roundtrip(gpu):
    """scafes_host_alloc memory (huge-page pinned) as the host side of
    upload and download: the same results as pageable numpy arrays."""
    M = gpu
    n = (40, 33, 29)
    shape = (n[2], n[1], n[0])
    u0 = np.random.default_rng(4).uniform(-1.0, 1.0, shape)
    cfg = M.make_cfg(n, tau=1e-4, heat=(1.0, 1.0, 0.0))
    with M.HostArray(shape) as hin, M.HostArray(shape) as hout:
        assert hin.p.value % 4096 == 0 and np.all(hin.a == 0.0)
        hin.a[...] = u0
        with M.Plain(cfg) as p:
            p.upload(M.FIELD_U, hin.a)
            p.step(7)
            p.download(M.FIELD_U, hout.a)
            ref = p.download()
        assert np.array_equal(hout.a, ref)


@pytest.mark.parametrize("prec", ["f64", "f32x2", "f32"])
def test_async_copies_on_two_handles(gpu, prec):
    """scafes_gpu_upload_async / _download_async / _synchronize, pipelined
    over two handles on two streams as the bench's end-to-end loop runs
    them: every step's result equals the synchronous path's bit for bit."""
    import torch
    M = gpu
    n = (48, 40, 36)
    shape = (n[2], n[1], n[0])
    rng = np.random.default_rng(9)
    inputs = [rng.uniform(-1.0, 1.0, shape) for _ in range(5)]
    cfg = dict(tau=1e-4, heat=(1.0, 1.0, 0.0), precision=prec)
    want = []
    with M.Plain(M.make_cfg(n, **cfg)) as p:
        for u in inputs:
            p.upload(M.FIELD_U, u)
            p.step(6)
            want.append(p.download())
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    hin = [M.HostArray(shape) for _ in range(2)]
    hout = [M.HostArray(shape) for _ in range(2)]
    got = [None] * len(inputs)
    handles = [M.Plain(M.make_cfg(n, stream=s.cuda_stream, **cfg)) for s in streams]
    try:
        for k, u in enumerate(inputs):
            h = handles[k % 2]
            if k >= 2:
                h.synchronize()
                got[k - 2] = hout[k % 2].a.copy()
            hin[k % 2].a[...] = u
            h.upload_async(hin[k % 2].a)
            h.step(6)
            h.download_async(hout[k % 2].a)
        for k in range(len(inputs) - 2, len(inputs)):
            handles[k % 2].synchronize()
            got[k] = hout[k % 2].a.copy()
    finally:
        for h in handles:
            h.close()
        for a in hin + hout:
            a.close()
    for k in range(len(inputs)):
        assert np.array_equal(got[k], want[k]), k
    with M.Plain(M.make_cfg(n, **cfg)) as p:
        with pytest.raises(M.ScafesError):
            p.download_async(np.empty(shape))  # nothing uploaded yet
        with pytest.raises(ValueError):
            p.upload_async(np.empty((3, 3)))
