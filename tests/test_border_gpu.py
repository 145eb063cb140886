"""Flux-condition borders (SCAFES_BORDER_TABLE) on the GPU against the oracle.

The reference's Neumann and Cauchy system tests (heat and Pennes,
TimeLinSpaceLin) run through the C ABI with the rules of
scafes_border_forms_flux and their known fields in the affine-in-time form
the device stores; the results must match the oracle (bit-exact to the
reference on these cases) to 1e-12 relative max-norm in FP64 and f32x2,
2e-5 in FP32.  A seeded case with noisy data and a non-cubic grid checks
more than linear solutions.
"""
from __future__ import annotations

import numpy as np
import pytest

import cases
import oracle as O
from test_oracle_golden import flux_case, radiation_case

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-12, "f32x2": 1e-12, "f32": 2e-5}


def affine(known, S_shape, time_fn=None):
    """(base, form, a, b) oracle known field -> (A, B) with K(t) = A + t B."""
    base, form, a, b = known
    base = np.broadcast_to(base, S_shape)
    if form == 0:
        return base * a, base * b
    if form == 1:
        return base * a + b * base, b * base
    if form == 2:
        return base * a + b, base * a + b
    raise ValueError(form)


def run_table(M, g, n, u0, T, kind, f, g_dir, g_flux, prec, heat, lam=1.0, alpha=1.0, n_layers=1):
    cfg = M.make_cfg(n, tau=g.tau, precision=prec, border=M.BORDER_TABLE, heat=heat, n_layers=n_layers)
    forms = M.border_forms_flux(cfg, kind, lam, alpha)
    shape = (n[2], n[1], n[0])
    fa, fb = affine(f, shape)
    # One border field G: Dirichlet values on min-face nodes, flux values on
    # the others (the reference's knownDf(1)).
    x0 = np.zeros(shape, dtype=bool)
    x0[:, :, 0] = x0[:, 0, :] = x0[0, :, :] = True
    ga_d, gb_d = affine(g_dir, shape)
    ga_f, gb_f = affine(g_flux, shape)
    ga = np.where(x0, ga_d, ga_f)
    gb = np.where(x0, gb_d, gb_f)
    with M.Plain(cfg) as p:
        p.set_border_forms(forms)
        p.upload(M.FIELD_F_A, fa)
        if np.any(fb):
            p.upload(M.FIELD_F_B, fb)
        p.upload(M.FIELD_G_A, ga)
        p.upload(M.FIELD_G_B, gb)
        p.upload(M.FIELD_U, u0)
        p.step(T)
        return p.download()


@pytest.mark.parametrize("name", ["heat_neumann", "heat_cauchy", "pennes_neumann", "pennes_cauchy",
                                  "heat_neumann_10x8x6"])
@pytest.mark.parametrize("prec", ["f64", "f32x2", "f32"])
def test_flux_border_golden(gpu, name, prec):
    M = gpu
    d, g, S, T, kind, f, g_flux, perf = flux_case(name)
    n = tuple(d["n"])
    heat = (1.0, 1.0, perf.get("perf_q1", 0.0) * perf.get("perf_w", 0.0))
    u = run_table(M, g, n, S * 1.0, T, kind, f, (S, 0, 1.0, 1.0), g_flux, prec, heat)
    assert cases.rel_err(u, d["final"]) <= TOL[prec], (name, prec)


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("prec", ["f64", "f32x2"])
def test_flux_border_noisy(gpu, kind, prec):
    M = gpu
    n, T = (37, 21, 19), 60
    rng = np.random.default_rng(40 + kind)
    shape = (n[2], n[1], n[0])
    h2 = sum(1.0 / ((1.0 / (m - 1)) ** 2) for m in n)
    tau = 0.8 / (2.0 * h2 * 1.3)
    g = O.make_grid(n, tau=tau)
    u0 = rng.uniform(-1.0, 1.0, shape)
    fb = rng.uniform(-1.0, 1.0, shape)
    gdir = rng.uniform(-1.0, 1.0, shape)
    gflx = rng.uniform(-1.0, 1.0, shape)
    coeff_a, lam, alpha = 1.3, 0.8, 0.6
    f = (fb, 0, 2.0, 0.5)
    ref = O.heat_flux(g, u0, T, kind, coeff_a=coeff_a, lam=lam, alpha=alpha, f=f,
                      g_dir=(gdir, 0, 1.0, -0.5), g_flux=(gflx, 0, 0.5, 1.5))
    u = run_table(M, g, n, u0, T, kind, f, (gdir, 0, 1.0, -0.5), (gflx, 0, 0.5, 1.5), prec,
                  (coeff_a, 1.0, 0.0), lam=lam, alpha=alpha)
    assert cases.rel_err(u, ref) <= 1e-12, (kind, prec)


# FP32 storage: one rounding of u (relative 6e-8, values up to 16) per step,
# forgotten at the slowest diffusion rate (about 3 pi^2 per unit time, 6e-4
# per step here) -- a worst-case bias bound of 3e-8 / 6e-4 = 5e-5.
RAD_TOL = {"f64": 1e-12, "f32x2": 1e-12, "f32": 1e-4}


def radiation_g(S, x0, t_center, t_rate):
    """Coefficients G_A .. G_E in s = (t - t_center) * t_rate of the border
    field of Radiation/TimeLinSpaceLin: S (1 + t) on min-face nodes,
    S^4 (1 + t)^4 + (1 + t) elsewhere; 1 + t = A + B s."""
    A, B = 1.0 + t_center, 1.0 / t_rate
    binom = (1, 4, 6, 4, 1)
    co = [S ** 4 * (binom[k] * A ** (4 - k) * B ** k) for k in range(5)]
    co[0] = co[0] + A
    co[1] = co[1] + B
    dirichlet = [S * A, S * B, 0.0 * S, 0.0 * S, 0.0 * S]
    return [np.where(x0, d, c) for d, c in zip(dirichlet, co)]


@pytest.mark.parametrize("name", ["pennes_radiation", "pennes_radiation_10x8x6"])
@pytest.mark.parametrize("basis", [(0.0, 1.0), (0.5, 2.0)])
@pytest.mark.parametrize("prec", ["f64", "f32x2", "f32"])
def test_radiation_border_golden(gpu, name, basis, prec):
    """The reference's Radiation system test: u^4 flux weights from
    scafes_border_forms_flux, the quartic-in-time border field as G_A .. G_E
    in the time basis `basis`, against the reference's own final iterate."""
    d, g, S, T = radiation_case(name)
    u = run_radiation(gpu, d, g, S, T, basis, prec)
    assert np.all(np.isfinite(u))
    assert cases.rel_err(u, d["final"]) <= RAD_TOL[prec], (name, basis, prec)


def run_radiation(M, d, g, S, T, basis, prec, n_layers=1):
    n = tuple(d["n"])
    shape = (n[2], n[1], n[0])
    cfg = M.make_cfg(n, tau=g.tau, precision=M.PRECISIONS[prec], border=M.BORDER_TABLE, heat=(1.0, 1.0, 1.0),
                     n_layers=n_layers)
    forms = M.border_forms_flux(cfg, M.FLUX_RADIATION, 1.0, 1.0)
    x0 = np.zeros(shape, dtype=bool)
    x0[:, :, 0] = x0[:, 0, :] = x0[0, :, :] = True
    fa, fb = affine((S, 1, 1.0, 1.0), shape)
    with M.Plain(cfg) as p:
        p.set_border_forms(forms)
        p.set_border_time_basis(*basis)
        p.upload(M.FIELD_F_A, fa)
        p.upload(M.FIELD_F_B, fb)
        for slot, c in zip((M.FIELD_G_A, M.FIELD_G_B, M.FIELD_G_C, M.FIELD_G_D, M.FIELD_G_E),
                           radiation_g(S, x0, *basis)):
            p.upload(slot, c)
        p.upload(M.FIELD_U, S * 1.0)
        p.step(T)
        return p.download()


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
def test_radiation_border_noisy(gpu, prec):
    """Seeded data on a non-cubic grid (37 x 21 x 19): random iterate,
    source and border field base, lambda, epsilon*sigma != 1, the radiation
    field (base (1 + t))^4 a + b (1 + t) as G_A .. G_E in the default time
    basis; against the oracle's restatement of Radiation.hpp (1e-12)."""
    M = gpu
    n, T = (37, 21, 19), 80
    rng = np.random.default_rng(61)
    shape = (n[2], n[1], n[0])
    h2 = sum((m - 1) ** 2 for m in n)
    tau = 0.3 / (2.0 * h2)
    g = O.make_grid(n, tau=tau)
    u0 = rng.uniform(0.5, 1.5, shape)
    fb = rng.uniform(-1.0, 1.0, shape)
    base = rng.uniform(0.5, 1.5, shape)
    gdir = rng.uniform(-1.0, 1.0, shape)
    lam, eps, sig, a, b = 0.8, 0.7, 0.9, 0.6, 1.3
    ref = O.heat_radiation(g, u0, T, coeff_a=1.1, lam=lam, epsilon=eps, sigma=sig, f=(fb, 0, 1.0, 0.0),
                           g_dir=(gdir, 0, 1.0, 0.0), g_flux=(base, 3, a, b))
    cfg = M.make_cfg(n, tau=tau, precision=prec, border=M.BORDER_TABLE, heat=(1.1, 1.0, 0.0))
    forms = M.border_forms_flux(cfg, M.FLUX_RADIATION, lam, eps * sig)
    x0 = np.zeros(shape, dtype=bool)
    x0[:, :, 0] = x0[:, 0, :] = x0[0, :, :] = True
    binom = (1, 4, 6, 4, 1)
    co = [a * base ** 4 * binom[k] for k in range(5)]   # (base (1+t))^4 a in powers of t
    co[0] = co[0] + b
    co[1] = co[1] + b
    zero = np.zeros(shape)
    gco = [np.where(x0, gdir, co[0])] + [np.where(x0, zero, c) for c in co[1:]]
    with M.Plain(cfg) as p:
        p.set_border_forms(forms)
        p.upload(M.FIELD_F_A, fb)
        for slot, c in zip((M.FIELD_G_A, M.FIELD_G_B, M.FIELD_G_C, M.FIELD_G_D, M.FIELD_G_E), gco):
            p.upload(slot, c)
        p.upload(M.FIELD_U, u0)
        p.step(T)
        u = p.download()
    assert cases.rel_err(u, ref) <= 1e-12, prec


def test_border_time_basis_rules(gpu):
    """Higher time orders of G and a non-default basis are TABLE-only; a
    zero rate is refused."""
    M = gpu
    n = (8, 8, 8)
    dcfg = M.make_cfg(n, tau=1e-3, heat=(1.0, 1.0, 0.0))
    with M.Plain(dcfg) as p:
        p.upload(M.FIELD_U, np.zeros((8, 8, 8)))
        with pytest.raises(M.ScafesError):
            p.set_border_time_basis(0.0, 0.0)
        p.upload(M.FIELD_G_C, np.ones((8, 8, 8)))
        with pytest.raises(M.ScafesError):
            p.step(1)
    with M.Plain(dcfg) as p:
        p.upload(M.FIELD_U, np.zeros((8, 8, 8)))
        p.set_border_time_basis(1.0, 1.0)
        with pytest.raises(M.ScafesError):
            p.step(1)


def test_border_table_errors(gpu):
    M = gpu
    n = (8, 8, 8)
    cfg = M.make_cfg(n, tau=1e-3, border=M.BORDER_TABLE, heat=(1.0, 1.0, 0.0))
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_U, np.zeros((8, 8, 8)))
        with pytest.raises(M.ScafesError):
            p.step(1)                       # no rules set yet
        forms = M.border_forms_flux(cfg, M.FLUX_NEUMANN)
        bad = M.BorderForms()
        C = __import__("ctypes")
        C.memmove(bad, forms, C.sizeof(forms))
        bad[1].cn[0] = 0.5                  # class x==0 reading x-1
        with pytest.raises(M.ScafesError):
            p.set_border_forms(bad)
        p.set_border_forms(forms)
        with pytest.raises(M.ScafesError):
            p.step(1)                       # the rules read F, none uploaded
    dcfg = M.make_cfg(n, tau=1e-3, heat=(1.0, 1.0, 0.0))
    with M.Plain(dcfg) as p:
        with pytest.raises(M.ScafesError):
            p.set_border_forms(M.border_forms_flux(dcfg, M.FLUX_NEUMANN))
