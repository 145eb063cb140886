"""Multi-field leapfrog workloads (C ABI, CUDA) against their oracle
restatements (orc_lame, orc_yee), plus size-independent properties.
Tolerances: 1e-12 relative max-norm for FP64 and FP32 pairs, 1e-4 for
FP32 (Yee)."""
from __future__ import annotations

import numpy as np
import pytest

import cases
import oracle as O
from masterthesis_gb300 import workloads as W

pytestmark = pytest.mark.gpu

LAME = (1.0, 0.5, 1.0)  # lambda, mu, rho


def run_lame(M, n, T, u0, tau, prec="f64"):
    with M.MultiField(M.MF_LAME, n, tau, LAME, precision=prec) as mf:
        for c in range(3):
            mf.upload(c, u0[c])
            mf.upload(3 + c, u0[c])
        mf.step(T)
        return np.stack([mf.download(c) for c in range(3)]), np.stack([mf.download(3 + c) for c in range(3)])


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
@pytest.mark.parametrize("n", [(13, 11, 9), (40, 33, 35)])
def test_lame_matches_oracle(gpu, n, prec):
    M = gpu
    T = 30
    u0 = W.gaussian_bump_displacement(n, seed=3)
    tau = W.lame_tau(n)
    u, up = run_lame(M, n, T, u0, tau, prec)
    g = O.make_grid(n, tau=tau)
    ru, rup = O.lame(g, u0, u0, T, *LAME)
    assert cases.rel_err(u, ru) <= 1e-12
    assert cases.rel_err(up, rup) <= 1e-12


def test_lame_full_size_bounded(gpu):
    """384^3 (the Lame-Navier workload size), 20 steps: finite, border at 0,
    and the displacement stays bounded (no blow-up of the leapfrog scheme)."""
    M = gpu
    n, T = (384, 384, 384), 20
    u0 = W.gaussian_bump_displacement(n, seed=3)
    u, _ = run_lame(M, n, T, u0, W.lame_tau(n))
    assert np.all(np.isfinite(u))
    assert np.max(np.abs(u)) <= 2.0 * np.max(np.abs(u0))
    assert np.all(u[:, 0] == 0.0) and np.all(u[:, :, :, -1] == 0.0)


def yee_fields_zero(n):
    return np.zeros((6, n[2], n[1], n[0]))


@pytest.mark.parametrize("prec,tol,n", [("f64", 1e-12, (20, 18, 16)), ("f32", 1e-4, (20, 18, 16)),
                                        ("f32", 1e-4, (37, 29, 41)), ("f64", 1e-12, (37, 29, 41)),
                                        ("f32x2", 1e-12, (20, 18, 16)), ("f32x2", 1e-12, (37, 29, 41))])
def test_yee_matches_oracle(gpu, prec, tol, n):
    """FP32 runs the fused one-pass step (tiles, halos and z-chunks cut
    across these odd sizes), FP64 the two-kernel step."""
    M = gpu
    T = 80
    tau, src, par = W.yee_setup(n)
    with M.MultiField(M.MF_YEE, n, tau, par, precision=prec, src=src) as mf:
        mf.step(T)
        f = np.stack([mf.download(i) for i in range(6)])
    g = O.make_grid(n, tau=tau)
    ref = O.yee(g, yee_fields_zero(n), T, src, *par)
    assert np.max(np.abs(ref)) > 0.0
    assert cases.rel_err(f, ref) <= tol


def test_yee_f32_fused_matches_f64_at_256(gpu):
    """256^3, 60 steps: the fused FP32 step (8 z-chunks of 32 planes, 64
    column tiles per plane) against the FP64 two-kernel step, all six fields,
    1e-4 relative max-norm as for the small FP32 case."""
    M = gpu
    n, T = (256, 256, 256), 60
    tau, src, par = W.yee_setup(n)
    out = {}
    for prec in ("f32", "f64"):
        with M.MultiField(M.MF_YEE, n, tau, par, precision=prec, src=src) as mf:
            mf.step(T)
            out[prec] = np.stack([mf.download(i) for i in range(6)])
    assert np.max(np.abs(out["f64"])) > 0.0
    assert cases.rel_err(out["f32"], out["f64"]) <= 1e-4


def test_yee_energy_bounded_after_source(gpu):
    """After the pulse the PEC cavity holds its energy (leapfrog: conserved
    up to O(tau) oscillation) -- no growth."""
    M = gpu
    n = (48, 48, 48)
    tau, src, par = W.yee_setup(n)
    amp, t0, w, freq = par
    t_off = t0 + 4 * w
    T1 = int(np.ceil(t_off / tau)) + 10
    with M.MultiField(M.MF_YEE, n, tau, par, precision="f64", src=src) as mf:
        mf.step(T1)
        e1 = sum(float(np.sum(mf.download(i) ** 2)) for i in range(6))
        mf.step(200)
        e2 = sum(float(np.sum(mf.download(i) ** 2)) for i in range(6))
    assert e1 > 0.0
    assert e2 <= e1 * 1.05
    assert e2 >= e1 * 0.95


def test_pairs_at_full_size_track_f64(gpu):
    """Lame 384^3 x 10 steps and Yee 256^3 x 60 steps: the FP32-pair runs
    against the FP64 runs (relative max-norm 1e-12)."""
    M = gpu
    n = (384, 384, 384)
    u0 = W.gaussian_bump_displacement(n, seed=3)
    a, _ = run_lame(M, n, 10, u0, W.lame_tau(n), "f64")
    b, _ = run_lame(M, n, 10, u0, W.lame_tau(n), "f32x2")
    del u0
    assert cases.rel_err(b, a) <= 1e-12
    del a, b
    n, T = (256, 256, 256), 60
    tau, src, par = W.yee_setup(n)
    out = {}
    for prec in ("f64", "f32x2"):
        with M.MultiField(M.MF_YEE, n, tau, par, precision=prec, src=src) as mf:
            mf.step(T)
            out[prec] = np.stack([mf.download(i) for i in range(6)])
    assert np.max(np.abs(out["f64"])) > 0.0
    assert cases.rel_err(out["f32x2"], out["f64"]) <= 1e-12


def test_multifield_errors(gpu):
    M = gpu
    with pytest.raises(M.ScafesError):
        M.MultiField(M.MF_LAME, (8, 8, 8), 1e-3, LAME, precision="f32")
    with pytest.raises(M.ScafesError):
        M.MultiField(M.MF_YEE, (8, 8, 8), 1e-3, (1, 0, 1, 1), src=(9, 0, 0))
    with M.MultiField(M.MF_YEE, (8, 8, 8), 1e-3, (1, 0, 1, 1), src=(4, 4, 4)) as mf:
        with pytest.raises(M.ScafesError):
            mf.upload(6, np.zeros(512))
        with pytest.raises(M.ScafesError):
            mf.upload(0, np.zeros(5))
