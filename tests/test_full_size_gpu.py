"""The workloads at their full sizes against the CPU oracle (C ABI, CUDA).

The smaller parity tests pin every code path on golden vectors and ragged
shapes; these run the measured configurations themselves -- the large heat
solve (512^3 x 1000 steps), the Pennes ensemble (256 instances x 500 steps),
Lame-Navier at 384^3 and Yee at 512^3, the adjoint on the workload's
problem -- and compare each result with the oracle's restatement of the
reference's update on the same inputs, run on all host cores (about a
minute each for the heat solve and the ensemble).  Tolerances: relative
max-norm 1e-12 for FP64 and FP32 pairs, 1e-4 for FP32, 1e-11 / 1e-9
for the adjoint (FP64 / pairs), as in the small-size tests.
"""
from __future__ import annotations

import os

import numpy as np
import pytest

import cases
import oracle as O
from masterthesis_gb300 import workloads as W

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module")
def heat512():
    """The large heat workload: 512^3, sine mode + seeded (seed 2) noise at
    inner nodes, Dirichlet 0, tau = 0.9 h^2/6, 1000 steps; initial iterate
    and the oracle's final iterate."""
    n, T = (512, 512, 512), 1000
    tau = W.heat_tau(n)
    u0 = W.heat_sine_noise(n, seed=2)
    g = O.make_grid(n, tau=tau)
    u = O.first_touched(u0.shape, THREADS)
    w = O.first_touched(u0.shape, THREADS)
    u[...] = u0
    ref = O.heat_dirichlet_ws(g, u, w, T, nthreads=THREADS)
    return n, T, tau, u0, ref.copy()


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
def test_config2_heat_512_matches_oracle(gpu, heat512, prec):
    """512^3 x 1000 steps: the FP64 sweep and the compensated FP32-pair
    sweep against the oracle, 1e-12; the maximum principle holds."""
    M = gpu
    n, T, tau, u0, ref = heat512
    cfg = M.make_cfg(n, tau=tau, precision=prec, heat=(1.0, 1.0, 0.0))
    u = cases.run(cfg, {M.FIELD_U: u0}, T)
    assert cases.rel_err(u, ref) <= 1e-12
    assert np.all(np.abs(u) <= np.max(np.abs(u0)) * (1 + 1e-12))


def test_config2_heat_512_f32_near_oracle(gpu, heat512):
    """Plain FP32 storage and arithmetic on the same solve: its error
    against the oracle is the FP32 rounding accumulated over 1000 steps
    (measured 3.4e-5 against the FP64 sweep; bound 1e-4)."""
    M = gpu
    n, T, tau, u0, ref = heat512
    cfg = M.make_cfg(n, tau=tau, precision="f32", heat=(1.0, 1.0, 0.0))
    assert cases.rel_err(cases.run(cfg, {M.FIELD_U: u0}, T), ref) <= 1e-4


@pytest.fixture(scope="module")
def ensemble():
    """The Pennes ensemble workload: 256 instances (seed 8), 500 steps; the
    oracle's final iterate of every instance."""
    specs = W.pennes_ensemble(n_inst=256, seed=8)
    T = 500
    refs = []
    for sp in specs:
        n = sp["n"]
        g = O.make_grid(n, tau=sp["tau"])
        u0 = np.full((n[2], n[1], n[0]), W.T_ARTERIAL)
        refs.append(O.pennes_mri(g, u0, T, 1.0, 1.0, sp["k"], 1.0, 1.0, sp["w_b"], W.T_ARTERIAL, sp["q"], u0,
                                 nthreads=THREADS))
    return specs, T, refs


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
def test_config5_ensemble_matches_oracle(gpu, ensemble, prec):
    """All 256 instances through the persistent work-queue kernel, the time
    loop replayed from its CUDA graph (autotuned schedule), each instance
    against the oracle, 1e-12 -- the FP32-pair path in its deviation form
    included."""
    M = gpu
    specs, T, refs = ensemble
    with M.Batch([W.pennes_batch_instance(s) for s in specs], precision=prec) as b:
        for i, s in enumerate(specs):
            b.upload(i, M.FIELD_F_A, W.pennes_source(s))
            b.upload(i, M.FIELD_U, np.full((s["n"][2], s["n"][1], s["n"][0]), W.T_ARTERIAL))
        b.autotune(3)
        for i, s in enumerate(specs):  # autotune restores the iterates; start again regardless
            b.upload(i, M.FIELD_U, np.full((s["n"][2], s["n"][1], s["n"][0]), W.T_ARTERIAL))
        b.step(T // 2)
        b.step(T - T // 2)   # a second graph replay of another length
        worst = max(cases.rel_err(b.download(i), refs[i]) for i in range(len(specs)))
    assert worst <= 1e-12, worst


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
def test_config3_lame_384_matches_oracle(gpu, prec):
    """Lame-Navier at its workload size, 384^3, 10 leapfrog steps from the
    seeded bump: both time levels against the oracle, 1e-12 (FP64 and FP32
    pairs)."""
    M = gpu
    n, T = (384, 384, 384), 10
    u0 = W.gaussian_bump_displacement(n, seed=3)
    tau = W.lame_tau(n)
    with M.MultiField(M.MF_LAME, n, tau, (1.0, 0.5, 1.0), precision=prec) as mf:
        for c in range(3):
            mf.upload(c, u0[c])
            mf.upload(3 + c, u0[c])
        mf.step(T)
        u = np.stack([mf.download(c) for c in range(3)])
        up = np.stack([mf.download(3 + c) for c in range(3)])
    ru, rup = O.lame(O.make_grid(n, tau=tau), u0, u0, T, 1.0, 0.5, 1.0, nthreads=THREADS)
    assert cases.rel_err(u, ru) <= 1e-12
    assert cases.rel_err(up, rup) <= 1e-12


@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f32x2", 1e-12), ("f32", 1e-4)])
def test_config3_yee_512_matches_oracle(gpu, prec, tol):
    """Yee FDTD at its workload size, 512^3, 20 steps of the seeded dipole
    from zero fields: all six fields against the oracle."""
    M = gpu
    n, T = (512, 512, 512), 20
    tau, src, par = W.yee_setup(n)
    with M.MultiField(M.MF_YEE, n, tau, par, precision=prec, src=src) as mf:
        mf.step(T)
        f = np.stack([mf.download(i) for i in range(6)])
    ref = O.yee(O.make_grid(n, tau=tau), np.zeros((6, 512, 512, 512)), T, src, *par, nthreads=THREADS)
    assert np.max(np.abs(ref)) > 0.0
    assert cases.rel_err(f, ref) <= tol


@pytest.mark.parametrize("prec,tol", [("f64", 1e-11), ("f32x2", 1e-9)])
def test_config4_adjoint_64_matches_oracle(gpu, prec, tol):
    """The adjoint workload's problem (k = exp(0.3 g), g a smoothed seeded
    Gaussian field, seed 5; target from k of seed 6; sine initial iterate)
    at 64^3 x 200 steps with 12 snapshots: J, dJ/dk and dJ/du0 against the
    oracle's adjoint, which stores every forward state."""
    M = gpu
    n, T = (64, 64, 64), 200

    def smooth(seed):
        g = np.random.default_rng(seed).standard_normal((n[2], n[1], n[0]))
        for _ in range(3):
            g[1:-1, 1:-1, 1:-1] = (g[2:, 1:-1, 1:-1] + g[:-2, 1:-1, 1:-1] + g[1:-1, 2:, 1:-1]
                                   + g[1:-1, :-2, 1:-1] + g[1:-1, 1:-1, 2:] + g[1:-1, 1:-1, :-2]) / 6.0
        return g

    k, k2 = np.exp(0.3 * smooth(5)), np.exp(0.3 * smooth(6))
    tau = 0.9 / (2.0 * max(k.max(), k2.max()) * sum((m - 1) ** 2 for m in n))
    u0 = W.heat_sine_noise(n, amp=0.0)
    g = O.make_grid(n, tau=tau)
    target = O.kheat_forward(g, k2, u0, T, nthreads=THREADS)
    _, traj = O.kheat_forward(g, k, u0, T, keep_traj=True, nthreads=THREADS)
    J_ref, gk_ref, gu_ref = O.kheat_adjoint(g, k, traj, target, nthreads=THREADS)
    with M.Adjoint(n, tau, 12, precision=prec) as a:
        a.set_conductivity(k)
        J, gk, gu = a.gradient(u0, target, T)
    assert abs(J - J_ref) <= tol * abs(J_ref)
    assert cases.rel_err(gk, gk_ref) <= tol
    assert cases.rel_err(gu, gu_ref) <= tol
