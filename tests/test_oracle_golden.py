"""The CPU oracle against the golden vectors made by the reference itself.

The golden vectors (tests/golden/, made by make_golden.py) are the final
iterates of the reference's own Problem::iterateOverTime() on its system-test
problems.  The C restatement must reproduce them bit for bit.  Where the
reference-driver programs are built (oracle/_ref, this container only), a
fresh reference run at another size is compared too.
"""
from __future__ import annotations

import tempfile

import numpy as np
import pytest

import oracle as O
from conftest import load_golden


def test_stencil_width_one_bit_exact():
    d = load_golden("stencil_width_one")
    n, T = tuple(d["n"]), int(d["nsteps"])
    g = O.make_grid(n, last=tuple(d["last"]), tau=1.0 / T)
    k, j, i = np.meshgrid(*(np.arange(v) for v in n[::-1]), indexing="ij")
    u = O.stencil_width_one(g, (i + j + k).astype(np.float64), T)
    assert np.array_equal(u, d["final"])
    # HeatEqnFdmStencilWidthOne.hpp:39-40: f^n = 2^n (i+j+k) exactly.
    assert np.array_equal(u, 2.0 ** T * (i + j + k))


def test_stencil_width_var_bit_exact():
    d = load_golden("stencil_width_var")
    n, T = tuple(d["n"]), int(d["nsteps"])
    g = O.make_grid(n, tau=1.0 / T)
    k, j, i = np.meshgrid(*(np.arange(v) for v in n[::-1]), indexing="ij")
    u0 = (i + j + k).astype(np.float64)
    for bw in range(3):
        u = O.stencil_width_var(g, u0, bw, T)
        assert np.array_equal(u, d["final"][bw])
        assert np.array_equal(u, u0 + 2.0 * T)  # exact solution i+j+k+2n


@pytest.mark.parametrize("name,pennes", [("heat_timelin", False), ("pennes_timelin", True)])
def test_timelin_bit_exact(name, pennes):
    d = load_golden(name)
    n, T = tuple(d["n"]), int(d["nsteps"])
    g = O.make_grid(n, tau=float(d["t_end"]) / T)
    x, y, z = O.coords(g)
    S = np.broadcast_to(((1.0 + x) + y) + z, (n[2], n[1], n[0])).copy()
    if pennes:
        u = O.heat_dirichlet(g, S * 1.0, T, perf_q1=1.0, perf_w=1.0, f_base=S, f_form=1,
                             f_a=1.0, f_b=1.0, g_base=S, g_a=1.0, g_b=1.0)
    else:
        u = O.heat_dirichlet(g, S * 1.0, T, f_base=S, g_base=S, g_a=1.0, g_b=1.0)
    assert np.array_equal(u, d["final"])
    exact = S * (1.0 + O.lib().orc_time(g, T))
    assert np.max(np.abs(u - exact)) / np.max(np.abs(exact)) < 1e-14


@pytest.mark.parametrize("name", ["heat_noise_16", "heat_noise_odd"])
def test_heat_noise_bit_exact(name):
    d = load_golden(name)
    n, T = tuple(d["n"]), int(d["nsteps"])
    g = O.make_grid(n, tau=float(d["tau"]))
    assert np.array_equal(O.heat_dirichlet(g, d["u0"], T), d["final"])


def test_pennes_mri_bit_exact():
    d = load_golden("pennes_mri")
    n, T = tuple(d["n"]), int(d["nsteps"])
    g = O.make_grid(n, tau=float(d["tau"]))
    u = O.pennes_mri(g, d["u0"], T, *d["params"], d["q"], d["g"])
    assert np.array_equal(u, d["final"])


def test_oracle_threads_deterministic():
    d = load_golden("heat_noise_16")
    g = O.make_grid(tuple(d["n"]), tau=float(d["tau"]))
    a = O.heat_dirichlet(g, d["u0"], 20, nthreads=1)
    b = O.heat_dirichlet(g, d["u0"], 20, nthreads=4)
    assert np.array_equal(a, b)


@pytest.mark.skipif(not O.ref_available("ref_heat_dirichlet"),
                    reason="reference-driver programs not built here (oracle/_ref)")
def test_fresh_reference_run_other_size():
    n, T = (11, 13, 7), 25
    h2 = sum((m - 1) ** 2 for m in n)
    tau = 0.9 / (2.0 * h2)
    g = O.make_grid(n, tau=tau)
    rng = np.random.default_rng(11)
    u0 = rng.uniform(-1, 1, (n[2], n[1], n[0]))
    u0[O.border_mask(g)] = 0.0
    with tempfile.TemporaryDirectory() as tmp:
        r = O.run_ref("ref_heat_dirichlet", n, T, tmp, tau=tau, t_end=tau * T, inputs=u0)
    assert np.array_equal(O.heat_dirichlet(g, u0, T), r)


def test_kheat_adjoint_matches_finite_differences():
    """The oracle's own adjoint (no reference counterpart: the reference
    only has ADOL-C forward mode) against central differences."""
    n, T = (9, 8, 7), 12
    h2 = sum((m - 1) ** 2 for m in n)
    g = O.make_grid(n, tau=0.2 / (2.0 * h2))
    rng = np.random.default_rng(5)
    shape = (n[2], n[1], n[0])
    k = np.exp(0.3 * rng.standard_normal(shape))
    u0 = rng.uniform(-1, 1, shape)
    target = rng.uniform(-1, 1, shape)
    _, traj = O.kheat_forward(g, k, u0, T, keep_traj=True)
    J, gk, gu = O.kheat_adjoint(g, k, traj, target)

    def J_of(kk, uu):
        uT = O.kheat_forward(g, kk, uu, T)
        return 0.5 * float(np.sum((uT - target) ** 2))

    assert abs(J - J_of(k, u0)) <= 1e-12 * abs(J)
    for seed in range(3):
        dk = np.random.default_rng(100 + seed).standard_normal(shape)
        du = np.random.default_rng(200 + seed).standard_normal(shape)
        eps = 1e-6
        fd_k = (J_of(k + eps * dk, u0) - J_of(k - eps * dk, u0)) / (2 * eps)
        fd_u = (J_of(k, u0 + eps * du) - J_of(k, u0 - eps * du)) / (2 * eps)
        assert abs(fd_k - np.sum(gk * dk)) <= 1e-6 * max(abs(fd_k), 1e-12)
        assert abs(fd_u - np.sum(gu * du)) <= 1e-6 * max(abs(fd_u), 1e-12)


def test_kheat_adjoint_matches_forward_mode_ad():
    """The oracle's adjoint against forward-mode AD of the forward solve (a
    dual-number restatement: the reference's ADOL-C gradient path is forward
    vector mode, fov_forward, and ADOL-C is not available here).  Exact
    derivatives on both sides: agreement to rounding, 1e-11 relative, at
    32^3 -- the size the reference's gradient is quoted at."""
    n, T = (32, 32, 32), 20
    h2 = sum((m - 1) ** 2 for m in n)
    g = O.make_grid(n, tau=0.4 / (2.0 * h2))
    rng = np.random.default_rng(7)
    shape = (n[2], n[1], n[0])
    k = np.exp(0.3 * rng.standard_normal(shape))
    u0 = rng.uniform(-1, 1, shape)
    target = rng.uniform(-1, 1, shape)
    _, traj = O.kheat_forward(g, k, u0, T, keep_traj=True)
    _, gk, gu = O.kheat_adjoint(g, k, traj, target)
    for seed in range(2):
        dk = np.random.default_rng(300 + seed).standard_normal(shape)
        du0 = np.random.default_rng(400 + seed).standard_normal(shape)
        uT, duT = O.kheat_tangent(g, k, dk, u0, du0, T)
        assert np.array_equal(uT, traj[-1])  # the value part is the forward solve
        dJ = float(np.sum((uT - target) * duT))
        adj = float(np.sum(gk * dk) + np.sum(gu * du0))
        assert abs(dJ - adj) <= 1e-11 * abs(dJ), (dJ, adj)


def flux_case(name):
    """Inputs of a flux-border TimeLinSpaceLin golden case (the known fields
    of tests/system/{HeatEqnFDM,PennesBioheatEqnFDM}/{Neumann,Cauchy}/
    TimeLinSpaceLin/TimeLinSpaceLin.hpp in the oracle's known-field forms)."""
    d = load_golden(name)
    n, T = tuple(d["n"]), int(d["nsteps"])
    g = O.make_grid(n, tau=float(d["t_end"]) / T)
    x, y, z = O.coords(g)
    S = np.broadcast_to(((1.0 + x) + y) + z, (n[2], n[1], n[0])).copy()
    pennes = name.startswith("pennes")
    kind = 1 if "cauchy" in name else 0
    f = (S, 1, 1.0, 1.0) if pennes else (S, 0, 1.0, 0.0)
    g_flux = (S, 2, 1.0, 1.0) if kind == 1 else (np.full(S.shape, -1.0), 0, 1.0, 1.0)
    perf = dict(perf_q1=1.0, perf_w=1.0) if pennes else {}
    return d, g, S, T, kind, f, g_flux, perf


def radiation_case(name):
    """Inputs of a radiation-border golden case (tests/system/
    PennesBioheatEqnFDM/Radiation/TimeLinSpaceLin/TimeLinSpaceLin.hpp: f as
    in the Pennes Dirichlet case, G = (1 + sum x)(1 + t) at min-face nodes
    and ((1 + sum x)(1 + t))^4 SIGMA EPSILON + LAMBDA (1 + t) elsewhere, with
    LAMBDA = SIGMA = EPSILON = 1)."""
    d = load_golden(name)
    n, T = tuple(d["n"]), int(d["nsteps"])
    g = O.make_grid(n, tau=float(d["t_end"]) / T)
    x, y, z = O.coords(g)
    S = np.broadcast_to(((1.0 + x) + y) + z, (n[2], n[1], n[0])).copy()
    return d, g, S, T


@pytest.mark.parametrize("name", ["pennes_radiation", "pennes_radiation_10x8x6"])
def test_radiation_border_bit_exact(name):
    d, g, S, T = radiation_case(name)
    u = O.heat_radiation(g, S * 1.0, T, perf_q1=1.0, perf_w=1.0, f=(S, 1, 1.0, 1.0), g_dir=(S, 0, 1.0, 1.0),
                         g_flux=(S, 3, 1.0, 1.0))
    assert np.array_equal(u, d["final"])
    exact = S * (1.0 + O.lib().orc_time(g, T))
    assert np.max(np.abs(u - exact)) / np.max(np.abs(exact)) < 1e-13


def layers_case(name):
    """Inputs of a golden case with nLayersAtBorder > 1: the TimeLinSpaceLin
    problems of HeatEqnFDM/Dirichlet, HeatEqnFDM/Neumann and
    PennesBioheatEqnFDM/Radiation with two or three border layers."""
    d = load_golden(name)
    n, T, nl = tuple(d["n"]), int(d["nsteps"]), int(d["n_layers"])
    g = O.make_grid(n, tau=float(d["t_end"]) / T, n_layers=nl)
    x, y, z = O.coords(g)
    S = np.broadcast_to(((1.0 + x) + y) + z, (n[2], n[1], n[0])).copy()
    return d, g, S, T, nl


def layers_oracle(name, g, S, T):
    if name.startswith("heat_timelin"):
        return O.heat_dirichlet(g, S * 1.0, T, f_base=S, g_base=S, g_a=1.0, g_b=1.0)
    if name.startswith("heat_neumann"):
        return O.heat_flux(g, S * 1.0, T, 0, f=(S, 0, 1.0, 0.0), g_dir=(S, 0, 1.0, 1.0),
                           g_flux=(np.full(S.shape, -1.0), 0, 1.0, 1.0))
    return O.heat_radiation(g, S * 1.0, T, perf_q1=1.0, perf_w=1.0, f=(S, 1, 1.0, 1.0), g_dir=(S, 0, 1.0, 1.0),
                            g_flux=(S, 3, 1.0, 1.0))


@pytest.mark.parametrize("name", ["heat_timelin_nl2", "heat_neumann_nl3", "pennes_radiation_nl2"])
def test_border_layers_bit_exact(name):
    d, g, S, T, nl = layers_case(name)
    u = layers_oracle(name, g, S, T)
    assert np.array_equal(u, d["final"])
    exact = S * (1.0 + O.lib().orc_time(g, T))
    assert np.max(np.abs(u - exact)) / np.max(np.abs(exact)) < 1e-13


@pytest.mark.parametrize("name", ["heat_neumann", "heat_cauchy", "pennes_neumann", "pennes_cauchy",
                                  "heat_neumann_10x8x6"])
def test_flux_border_bit_exact(name):
    d, g, S, T, kind, f, g_flux, perf = flux_case(name)
    u = O.heat_flux(g, S * 1.0, T, kind, f=f, g_dir=(S, 0, 1.0, 1.0), g_flux=g_flux, **perf)
    assert np.array_equal(u, d["final"])
    exact = S * (1.0 + O.lib().orc_time(g, T))
    assert np.max(np.abs(u - exact)) / np.max(np.abs(exact)) < 1e-14


@pytest.mark.parametrize("name", ["tissue_tumour", "tissue_mri_closed", "tissue_mri_open"])
def test_tissue_examples_bit_exact(name):
    """The oracle's restatement of the reference's tissue examples
    (examples/TumorHeatEqnFDM/TumorHeatEqnFDM.hpp:234-353, examples/
    MRIDataPBHEqnFDM/MRIDataPBHEqnFDM.hpp:143-275: coefficients per node,
    Neumann / Cauchy / radiation borders) against the reference's own classes
    run by its Problem::iterateOverTime, bit for bit."""
    import cases
    d, g, fields, kw, u0 = cases.tissue_case(name)
    u = O.pennes_tissue(g, u0, int(d["nsteps"]), fields, **kw)
    assert np.array_equal(u, d["final"])


def test_oracle_adjoint_matches_reference_dual_numbers():
    """The oracle's adjoint at k = 1 (the flux-form heat update with a
    uniform conductivity is the reference's heat update with COEFF_A = 1)
    against directional derivatives taken through the reference's own
    updateInner<TT>/updateBorder<TT> with a dual number
    (tests/golden/heat_tangent_32.npz, oracle/ref_harness/
    ref_heat_tangent.cpp): <dJ/du0, d_k> = dJ_k for four seeded directions,
    and the forward solve equals the reference's, to 1e-12."""
    import cases
    d = load_golden("heat_tangent_32")
    n = tuple(int(v) for v in d["n"])
    T, tau = int(d["nsteps"]), float(d["tau"])
    u0, target, dirs = cases.tangent_inputs(n)
    g = O.make_grid(n, tau=tau)
    k = np.ones_like(u0)
    uT, traj = O.kheat_forward(g, k, u0, T, keep_traj=True)
    assert np.max(np.abs(uT - d["uT"])) <= 1e-12 * np.max(np.abs(d["uT"]))
    _, _, gu = O.kheat_adjoint(g, k, traj, target)
    # The oracle's engine holds border nodes at u0's values, so its dJ/du0
    # agrees with the Dirichlet problem's on the inner nodes: directions
    # with a zero border.
    border = O.border_mask(g)
    for dk, ref in zip(dirs, d["dJ_inner"]):
        dk = np.where(border, 0.0, dk)
        got = float(np.sum(gu * dk))
        assert abs(got - ref) <= 1e-11 * float(np.sum(np.abs(gu * dk))), (got, ref)
    # With the border reset every step (the reference's Dirichlet border), the
    # whole dJ/du0 -- border nodes included -- is the reference's.
    _, _, gu = O.kheat_adjoint(g, k, traj, target, reset_border=True)
    for dk, ref in zip(dirs, d["dJ"]):
        got = float(np.sum(gu * dk))
        assert abs(got - ref) <= 1e-11 * float(np.sum(np.abs(gu * dk))), (got, ref)
