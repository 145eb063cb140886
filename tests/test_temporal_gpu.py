"""Temporal blocking (depth 2: one pass per two steps) against depth 1 on
the GPU: the pass evaluates the same per-node arithmetic, so the results
must be identical bit for bit -- for every element type, with and without a
static source, with an affine Dirichlet border field, odd step counts (the
last step runs depth 1), grids whose tiles, halos and z-chunks are ragged
(one CTA spans x0-2 .. x0+33), and the step counter and launch count of
the C ABI.  Also against the oracle, and the autotuner's choice."""
from __future__ import annotations

import numpy as np
import pytest

import cases
import oracle as O

pytestmark = pytest.mark.gpu


def run(M, n, T, prec, depth, src, seed=5, tau_frac=0.9):
    """Heat with a random iterate, a static source (src) and the Dirichlet
    border field G = gbase * (1 + 0.5 time); returns the final iterate, the
    launches of the step call and the inputs."""
    rng = np.random.default_rng(seed)
    shape = (n[2], n[1], n[0])
    h2 = sum((m - 1) ** 2 for m in n)
    tau = tau_frac / (2.0 * h2)
    u0 = rng.uniform(-1.0, 1.0, shape)
    gbase = rng.uniform(-1.0, 1.0, shape)
    fa = rng.uniform(-1.0, 1.0, shape)
    cfg = M.make_cfg(n, tau=tau, precision=prec, heat=(1.0, 1.0, 0.0))
    with M.Plain(cfg) as p:
        if src:
            p.upload(M.FIELD_F_A, fa)
        p.upload(M.FIELD_G_A, gbase)
        p.upload(M.FIELD_G_B, 0.5 * gbase)
        p.upload(M.FIELD_U, u0)
        p.set_temporal_depth(depth)
        assert p.temporal_depth == depth
        p.step(T)
        launches = p.last_step_launches()
        return p.download(), launches, (u0, fa if src else None, gbase, tau)


@pytest.mark.parametrize("prec", ["f64", "f32x2", "f32"])
@pytest.mark.parametrize("n,T", [((45, 37, 29), 9), ((70, 33, 50), 8), ((33, 17, 5), 3), ((3, 3, 3), 4)])
@pytest.mark.parametrize("src", [False, True])
def test_depth2_equals_depth1(gpu, prec, n, T, src):
    M = gpu
    u1, l1, _ = run(M, n, T, prec, 1, src)
    u2, l2, _ = run(M, n, T, prec, 2, src)
    assert np.array_equal(u1, u2), (prec, n, T, src)
    assert l1 == T and l2 == (T + 1) // 2


def test_depth2_matches_oracle(gpu):
    M = gpu
    n, T = (66, 40, 35), 20
    u, _, (u0, fa, gbase, tau) = run(M, n, T, "f64", 2, True)
    g = O.make_grid(n, tau=tau)
    ref = O.heat_dirichlet(g, u0, T, f_base=fa, f_a=1.0, f_b=0.0, g_base=gbase, g_a=1.0, g_b=0.5)
    assert cases.rel_err(u, ref) <= 1e-12


def test_depth_rules_and_autotune(gpu):
    M = gpu
    n = (64, 48, 40)
    cfg = M.make_cfg(n, tau=1e-5, precision="f32", heat=(1.0, 1.0, 0.0))
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_U, np.zeros((40, 48, 64)))
        with pytest.raises(M.ScafesError):
            p.set_temporal_depth(3)
        p.autotune(4)
        assert p.temporal_depth in (1, 2)
        p.upload(M.FIELD_F_A, np.zeros((40, 48, 64)))
        p.upload(M.FIELD_F_B, np.ones((40, 48, 64)))   # a time-dependent source: depth 1 only
        p.set_temporal_depth(2)
        assert p.temporal_depth == 1
    tcfg = M.make_cfg(n, tau=1e-5, precision="f64", border=M.BORDER_TABLE, heat=(1.0, 1.0, 0.0))
    with M.Plain(tcfg) as p:
        p.set_temporal_depth(2)
        assert p.temporal_depth == 1                      # rule-table border: depth 1 only
