"""Hand-written adjoint with binomial checkpointing.

CPU: the schedule's forward-step count against a brute-force dynamic
program.  GPU (C ABI): J, dJ/dk and dJ/du0 against the CPU oracle's adjoint
(itself checked against central differences in test_oracle_golden.py),
identical results for every snapshot count, and central finite differences
of J on seeded random directions computed with the GPU forward solve.
Tolerances: 1e-11 relative max-norm against the oracle (FP64, different
evaluation order); 1e-6 relative against central differences.
"""
from __future__ import annotations

import functools

import numpy as np
import pytest

import cases
import oracle as O


def brute_cost(n, s):
    @functools.lru_cache(maxsize=None)
    def c(nn, ss):
        if nn == 1:
            return 0
        if ss == 0:
            return nn * (nn - 1) // 2
        return min(m + c(nn - m, ss - 1) + c(m, ss) for m in range(1, nn))
    return c(n, min(s, n - 1)) + 1


@pytest.mark.parametrize("n,snaps", [(1, 2), (2, 2), (7, 2), (30, 3), (64, 5), (100, 8), (50, 51), (200, 12)])
def test_schedule_cost_matches_brute_force(native, n, snaps):
    assert native.Adjoint.schedule_cost(n, snaps) == brute_cost(n, snaps - 1)


def test_schedule_cost_closed_form_against_recursion(native):
    """The schedule's closed form against the recursion itself on a range
    of step and snapshot counts (the first tests cover the small corner),
    and snapshot counts far above the 128 the recursion once capped at."""
    N, S = 260, 40
    C = [[0] * (S + 1) for _ in range(N + 1)]
    for n in range(1, N + 1):
        C[n][0] = n * (n - 1) // 2
    for s in range(1, S + 1):
        for n in range(2, N + 1):
            C[n][s] = n - 1 if s >= n - 1 else min(m + C[n - m][s - 1] + C[m][s] for m in range(1, n))
    for s in (1, 2, 3, 7, 19, 40):
        for n in (2, 3, 17, 64, 129, 200, 260):
            assert native.Adjoint.schedule_cost(n, s + 1) == C[n][s] + 1 if s < n - 1 else n, (n, s)
    A = native.Adjoint
    costs = [A.schedule_cost(2000, s) for s in (45, 128, 256, 512, 1000, 2000)]
    assert all(a > b for a, b in zip(costs, costs[1:]))
    assert costs[-1] == 2000 and costs[0] == 4873


def test_schedule_cost_store_all_and_monotone(native):
    A = native.Adjoint
    assert A.schedule_cost(2000, 2000) == 2000
    costs = [A.schedule_cost(500, s) for s in (2, 3, 5, 10, 20, 45, 100, 500)]
    assert all(a >= b for a, b in zip(costs, costs[1:]))


def kheat_problem(n, T, seed):
    rng = np.random.default_rng(seed)
    shape = (n[2], n[1], n[0])
    g = rng.standard_normal(shape)
    for _ in range(3):  # smooth by Jacobi passes
        g[1:-1, 1:-1, 1:-1] = (g[2:, 1:-1, 1:-1] + g[:-2, 1:-1, 1:-1] + g[1:-1, 2:, 1:-1] + g[1:-1, :-2, 1:-1]
                               + g[1:-1, 1:-1, 2:] + g[1:-1, 1:-1, :-2]) / 6.0
    k = np.exp(0.3 * g)
    tau = 0.9 / (2.0 * k.max() * sum((m - 1) ** 2 for m in n))
    u0 = rng.uniform(-1.0, 1.0, shape)
    target = rng.uniform(-1.0, 1.0, shape)
    return k, tau, u0, target


@pytest.mark.gpu
def test_adjoint_matches_oracle_all_snapshot_counts(gpu):
    M = gpu
    n, T = (12, 10, 9), 30
    k, tau, u0, target = kheat_problem(n, T, 7)
    g = O.make_grid(n, tau=tau)
    _, traj = O.kheat_forward(g, k, u0, T, keep_traj=True)
    J_ref, gk_ref, gu_ref = O.kheat_adjoint(g, k, traj, target)
    first = None
    for snaps in (2, 3, 7, 31, 64):
        with M.Adjoint(n, tau, snaps) as a:
            a.set_conductivity(k)
            J, gk, gu = a.gradient(u0, target, T)
            st = a.stats()
        assert abs(J - J_ref) <= 1e-12 * abs(J_ref)
        assert cases.rel_err(gk, gk_ref) <= 1e-11, snaps
        assert cases.rel_err(gu, gu_ref) <= 1e-11, snaps
        assert st["adjoint_steps"] == T
        assert st["forward_steps"] == M.Adjoint.schedule_cost(T, snaps)
        if first is None:
            first = (gk, gu)
        else:
            assert np.array_equal(gk, first[0]) and np.array_equal(gu, first[1]), snaps


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f32x2"])
def test_adjoint_backward_with_cotangent(gpu, prec):
    """scafes_adj_backward (any dJ/du_T): with dJ/du_T = u_T - target it
    gives scafes_adj_gradient's results bit for bit; for a random cotangent s
    it is the vector-Jacobian product -- u_T is linear in u0, so
    <s, u_T(u0 + d) - u_T(u0)> = <dJ/du0, d> to 1e-10 relative -- and it
    matches the oracle's adjoint run with target u_T - s (1e-11 FP64,
    1e-10 f32x2, as the other oracle comparisons)."""
    M = gpu
    n, T = (16, 12, 10), 30
    k, tau, u0, target = kheat_problem(n, T, 21)
    rng = np.random.default_rng(22)
    s = rng.uniform(-1.0, 1.0, u0.shape)
    d = rng.uniform(-1.0, 1.0, u0.shape)
    with M.Adjoint(n, tau, 5, precision=prec) as a:
        a.set_conductivity(k)
        J, gk, gu = a.gradient(u0, target, T)
        uT = a.forward(u0, T)
        gk2, gu2 = a.backward(u0, uT - target, T)
        assert np.array_equal(gk, gk2) and np.array_equal(gu, gu2)
        gks, gus = a.backward(u0, s, T)
        duT = a.forward(u0 + d, T) - uT
    lhs, rhs = float(np.sum(s * duT)), float(np.sum(gus * d))
    assert abs(lhs - rhs) <= 1e-10 * np.sum(np.abs(s * duT)), (lhs, rhs)
    g = O.make_grid(n, tau=tau)
    uT_ref, traj = O.kheat_forward(g, k, u0, T, keep_traj=True)
    _, gk_ref, gu_ref = O.kheat_adjoint(g, k, traj, uT_ref - s)
    tol = 1e-11 if prec == "f64" else 1e-10
    assert cases.rel_err(gks, gk_ref) <= tol
    assert cases.rel_err(gus, gu_ref) <= tol


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("f64", 1e-11), ("f32x2", 1e-9)])
def test_adjoint_matches_forward_mode_ad_32(gpu, prec, tol):
    """The GPU gradient at 32^3 (checkpointed, 8 snapshots over 60 steps)
    against forward-mode AD of the forward solve on the CPU (dual numbers:
    the mode of the reference's ADOL-C gradient, which is not available):
    <dJ/dk, dk> + <dJ/du0, du0> = <u_T - target, du_T> on 4 seeded
    directions, to 1e-11 (FP64) and 1e-9 (pairs, whose gradient fields are
    within 1e-10 of FP64)."""
    M = gpu
    n, T = (32, 32, 32), 60
    k, tau, u0, target = kheat_problem(n, T, 13)
    with M.Adjoint(n, tau, 8, precision=prec) as a:
        a.set_conductivity(k)
        _, gk, gu = a.gradient(u0, target, T)
    g = O.make_grid(n, tau=tau)
    for seed in range(4):
        dk = np.random.default_rng(500 + seed).standard_normal(u0.shape)
        du0 = np.random.default_rng(600 + seed).standard_normal(u0.shape)
        uT, duT = O.kheat_tangent(g, k, dk, u0, du0, T)
        dJ = float(np.sum((uT - target) * duT))
        adj = float(np.sum(gk * dk) + np.sum(gu * du0))
        assert abs(dJ - adj) <= tol * abs(dJ), (seed, dJ, adj)


@pytest.mark.gpu
def test_adjoint_forward_matches_oracle(gpu):
    M = gpu
    n, T = (17, 9, 13), 25
    k, tau, u0, _ = kheat_problem(n, T, 3)
    g = O.make_grid(n, tau=tau)
    with M.Adjoint(n, tau, 2) as a:
        a.set_conductivity(k)
        uT = a.forward(u0, T)
    assert cases.rel_err(uT, O.kheat_forward(g, k, u0, T)) <= 1e-12


@pytest.mark.gpu
def test_adjoint_gradient_vs_central_differences(gpu):
    M = gpu
    n, T = (20, 18, 16), 40
    k, tau, u0, target = kheat_problem(n, T, 11)
    with M.Adjoint(n, tau, 6) as a:
        a.set_conductivity(k)
        J, gk, gu = a.gradient(u0, target, T)

        def J_of(kk, uu):
            a.set_conductivity(kk)
            uT = a.forward(uu, T)
            return 0.5 * float(np.sum((uT - target) ** 2))

        for seed in range(4):
            rng = np.random.default_rng(1000 + seed)
            dk = rng.standard_normal(k.shape) * k
            du = rng.standard_normal(k.shape)
            eps = 1e-6
            fd_k = (J_of(k + eps * dk, u0) - J_of(k - eps * dk, u0)) / (2 * eps)
            fd_u = (J_of(k, u0 + eps * du) - J_of(k, u0 - eps * du)) / (2 * eps)
            assert abs(fd_k - float(np.sum(gk * dk))) <= 1e-6 * abs(fd_k), seed
            assert abs(fd_u - float(np.sum(gu * du))) <= 1e-6 * abs(fd_u), seed


@pytest.mark.gpu
def test_adjoint_f32x2_matches_oracle_and_f64(gpu):
    """The compensated FP32-pair sweeps (diagonal form of the same update)
    against the FP64 oracle: forward state and gradients to 1e-10 relative
    max-norm (pair arithmetic carries ~48 bits; the diagonal form rounds
    differently from the flux form), J to 1e-11."""
    M = gpu
    n, T = (12, 10, 9), 30
    k, tau, u0, target = kheat_problem(n, T, 7)
    g = O.make_grid(n, tau=tau)
    uT_ref, traj = O.kheat_forward(g, k, u0, T, keep_traj=True)
    J_ref, gk_ref, gu_ref = O.kheat_adjoint(g, k, traj, target)
    for snaps in (2, 5, 64):
        with M.Adjoint(n, tau, snaps, precision="f32x2") as a:
            a.set_conductivity(k)
            uT = a.forward(u0, T)
            J, gk, gu = a.gradient(u0, target, T)
            st = a.stats()
        assert cases.rel_err(uT, uT_ref) <= 1e-11, snaps
        assert abs(J - J_ref) <= 1e-11 * abs(J_ref), snaps
        assert cases.rel_err(gk, gk_ref) <= 1e-10, snaps
        assert cases.rel_err(gu, gu_ref) <= 1e-10, snaps
        assert st["forward_steps"] == M.Adjoint.schedule_cost(T, snaps)


@pytest.mark.gpu
def test_adjoint_f32x2_several_tiles_match_oracle(gpu):
    """The pair steps march 32 x 8 column tiles over 32-plane chunks: a grid
    of 3 x 3 tiles and 3 chunks with ragged last tiles in every direction
    (one-column, three-row and one-plane remainders) against the FP64
    oracle at the same 1e-10 / 1e-11 bars."""
    M = gpu
    n, T = (65, 19, 65), 12
    k, tau, u0, target = kheat_problem(n, T, 17)
    g = O.make_grid(n, tau=tau)
    uT_ref, traj = O.kheat_forward(g, k, u0, T, keep_traj=True)
    J_ref, gk_ref, gu_ref = O.kheat_adjoint(g, k, traj, target)
    with M.Adjoint(n, tau, 4, precision="f32x2") as a:
        a.set_conductivity(k)
        uT = a.forward(u0, T)
        J, gk, gu = a.gradient(u0, target, T)
    assert cases.rel_err(uT, uT_ref) <= 1e-11
    assert abs(J - J_ref) <= 1e-11 * abs(J_ref)
    assert cases.rel_err(gk, gk_ref) <= 1e-10
    assert cases.rel_err(gu, gu_ref) <= 1e-10


@pytest.mark.gpu
def test_adjoint_f32x2_gradient_vs_central_differences(gpu):
    M = gpu
    n, T = (20, 18, 16), 40
    k, tau, u0, target = kheat_problem(n, T, 11)
    with M.Adjoint(n, tau, 6, precision="f32x2") as a:
        a.set_conductivity(k)
        J, gk, gu = a.gradient(u0, target, T)
    # The differences use FP64 forward solves: J's rounding noise in pair
    # arithmetic (~1e-13 relative) over 2 eps would swamp a 1e-6 check.
    with M.Adjoint(n, tau, 2) as a:

        def J_of(kk, uu):
            a.set_conductivity(kk)
            uT = a.forward(uu, T)
            return 0.5 * float(np.sum((uT - target) ** 2))

        for seed in range(4):
            rng = np.random.default_rng(2000 + seed)
            dk = rng.standard_normal(k.shape) * k
            du = rng.standard_normal(k.shape)
            eps = 1e-6
            fd_k = (J_of(k + eps * dk, u0) - J_of(k - eps * dk, u0)) / (2 * eps)
            fd_u = (J_of(k, u0 + eps * du) - J_of(k, u0 - eps * du)) / (2 * eps)
            assert abs(fd_k - float(np.sum(gk * dk))) <= 1e-6 * abs(fd_k), seed
            assert abs(fd_u - float(np.sum(gu * du))) <= 1e-6 * abs(fd_u), seed


@pytest.mark.gpu
def test_adjoint_rejects_unsupported_precision(gpu):
    M = gpu
    with pytest.raises(M.ScafesError):
        M.Adjoint((8, 8, 8), 1e-3, 2, precision="f32")


def plain_heat_case(n, T, a, seed):
    rng = np.random.default_rng(seed)
    shape = (n[2], n[1], n[0])
    tau = 0.9 / (2.0 * a * sum((m - 1) ** 2 for m in n))
    g = O.make_grid(n, tau=tau)
    u0 = rng.uniform(-1.0, 1.0, shape)
    u0[O.border_mask(g)] = 0.0
    return g, tau, u0, rng.uniform(-1.0, 1.0, shape)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("f64", 1e-11), ("f32x2", 1e-10)])
def test_plain_handle_backward_entry_matches_oracle(gpu, prec, tol):
    """scafes_gpu_adjoint on a plain heat handle (coefficient a, Dirichlet
    0): the forward iterate equals the flux-form solve with k = a, and the
    gradients for the cotangent u_T - target are the oracle's dJ/dk, dJ/du0
    of J = 0.5 |u_T - target|^2 at k = a, with 6 checkpoints over 25 steps
    (recomputation), then again with enough for every state."""
    M = gpu
    n, T, a = (20, 17, 15), 25, 0.7
    g, tau, u0, target = plain_heat_case(n, T, a, 31)
    k = np.full(u0.shape, a)
    uT_ref, traj = O.kheat_forward(g, k, u0, T, keep_traj=True)
    # The handle's border is a Dirichlet border (reset every step).
    _, gk_ref, gu_ref = O.kheat_adjoint(g, k, traj, target, reset_border=True)
    with M.Plain(M.make_cfg(n, tau=tau, precision=prec, heat=(a, 1.0, 0.0))) as p:
        p.keep_initial()
        p.upload(M.FIELD_U, u0)
        p.step(T)
        uT = p.download()
        for ckpt in (6, 32):
            gk, gu = p.adjoint(uT - target, ckpt)
            assert cases.rel_err(gk, gk_ref) <= tol, ckpt
            assert cases.rel_err(gu, gu_ref) <= tol, ckpt
    assert cases.rel_err(uT, uT_ref) <= (1e-12 if prec == "f64" else 1e-11)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("f64", 1e-11), ("f32x2", 1e-10)])
def test_plain_handle_backward_entry_nonzero_border(gpu, prec, tol):
    """A non-zero constant Dirichlet value: G_A uploaded as 0.35 everywhere
    and u0 equal to it on the border (the border check compares the two in
    the handle's arithmetic, FP32 pairs included); the forward iterate and
    both gradients against the oracle; then an initial iterate whose border
    differs from G_A is refused (UNSUPPORTED) and the handle still works."""
    M = gpu
    n, T, a, gval = (18, 16, 14), 20, 0.6, 0.35
    g, tau, u0, target = plain_heat_case(n, T, a, 41)
    u0[O.border_mask(g)] = gval
    k = np.full(u0.shape, a)
    uT_ref, traj = O.kheat_forward(g, k, u0, T, keep_traj=True)
    _, gk_ref, gu_ref = O.kheat_adjoint(g, k, traj, target, reset_border=True)
    with M.Plain(M.make_cfg(n, tau=tau, precision=prec, heat=(a, 1.0, 0.0))) as p:
        p.upload(M.FIELD_G_A, np.full(u0.shape, gval))
        p.keep_initial()
        p.upload(M.FIELD_U, u0)
        p.step(T)
        uT = p.download()
        gk, gu = p.adjoint(uT - target, 5)
        assert cases.rel_err(uT, uT_ref) <= (1e-12 if prec == "f64" else 1e-11)
        assert cases.rel_err(gk, gk_ref) <= tol
        assert cases.rel_err(gu, gu_ref) <= tol
        bad = u0.copy()
        bad[0, 3, 4] = gval + 0.25           # one border node off the Dirichlet value
        p.upload(M.FIELD_U, bad)
        p.step(T)
        with pytest.raises(M.ScafesError) as e:
            p.adjoint(p.download() - target, 5)
        assert e.value.code == -4
        p.upload(M.FIELD_U, u0)               # a valid run afterwards gives the same gradients
        p.step(T)
        gk2, gu2 = p.adjoint(p.download() - target, 5)
        assert np.array_equal(gk2, gk) and np.array_equal(gu2, gu)


@pytest.mark.gpu
def test_plain_handle_backward_entry_refuses_what_it_does_not_cover(gpu):
    """Status codes, no fault: no kept initial iterate or no step (STATE),
    a border that differs from the Dirichlet value, a source, the Pennes
    perfusion term or the mirror border (UNSUPPORTED); the handle still
    steps correctly afterwards."""
    M = gpu
    STATE, UNSUPPORTED = -3, -4
    n, T, a = (12, 10, 9), 6, 1.0
    g, tau, u0, target = plain_heat_case(n, T, a, 5)
    cot = np.ones(u0.shape)

    def code(p):
        with pytest.raises(M.ScafesError) as ex:
            p.adjoint(cot, 4)
        return ex.value.code

    with M.Plain(M.make_cfg(n, tau=tau, heat=(a, 1.0, 0.0))) as p:
        p.upload(M.FIELD_U, u0)
        p.step(T)
        assert code(p) == STATE                        # no kept initial iterate
        p.keep_initial()
        p.upload(M.FIELD_U, u0)
        assert code(p) == STATE                        # no step since the upload
        bad = u0.copy()
        bad[0, 0, 0] = 0.5
        p.upload(M.FIELD_U, bad)
        p.step(T)
        assert code(p) == UNSUPPORTED                  # border differs from G = 0
        p.upload(M.FIELD_U, u0)
        p.step(T)
        u = p.download()
    assert cases.rel_err(u, O.heat_dirichlet(g, u0, T)) <= 1e-12
    with M.Plain(M.make_cfg(n, tau=tau, heat=(a, 1.0, 0.0))) as p:
        p.keep_initial()
        p.upload(M.FIELD_F_A, np.ones(u0.shape))
        p.upload(M.FIELD_U, u0)
        p.step(T)
        assert code(p) == UNSUPPORTED                  # a source
    with M.Plain(M.make_cfg(n, tau=tau, heat=(a, 1.0, 0.3))) as p:
        p.keep_initial()
        p.upload(M.FIELD_U, u0)
        p.step(T)
        assert code(p) == UNSUPPORTED                  # perfusion: not the heat form


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("f64", 1e-10), ("f32x2", 1e-9)])
def test_plain_handle_gradient_matches_reference_dual_numbers(gpu, prec, tol):
    """dJ/du0 of scafes_gpu_adjoint on the heat problem at 32^3 x 60 steps
    (checkpointed, 8 snapshots) against directional derivatives taken
    through the reference's own updateInner<TT>/updateBorder<TT> with a dual
    number (tests/golden/heat_tangent_32.npz, made by oracle/ref_harness/
    ref_heat_tangent.cpp from the untouched reference headers):
    <dJ/du0, d_k> = dJ_k for four seeded directions over all nodes, border
    included (a border value enters the first step only: the Dirichlet
    border resets it)."""
    from conftest import load_golden
    M = gpu
    d = load_golden("heat_tangent_32")
    n = tuple(int(v) for v in d["n"])
    T, tau = int(d["nsteps"]), float(d["tau"])
    u0, target, dirs = cases.tangent_inputs(n)
    with M.Plain(M.make_cfg(n, tau=tau, precision=prec, heat=(1.0, 1.0, 0.0))) as p:
        p.keep_initial()
        p.upload(M.FIELD_U, u0)
        p.step(T)
        uT = p.download()
        _, gu = p.adjoint(uT - target, 8)
    assert cases.rel_err(uT, d["uT"]) <= (1e-12 if prec == "f64" else 1e-11)
    for dk, ref in zip(dirs, d["dJ"]):
        got = float(np.sum(gu * dk))
        assert abs(got - ref) <= tol * float(np.sum(np.abs(gu * dk))), (got, ref)
