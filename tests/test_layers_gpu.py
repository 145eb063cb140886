"""nLayersAtBorder > 1 on the GPU (src/ScaFES_Problem.hpp:3952-3971: a node
within n_layers of a face is a border node): the reference's Dirichlet,
Neumann and Radiation system tests run with two or three border layers
(golden vectors of the reference itself), and seeded noisy cases on grids
whose 32-wide tiles start inside and outside the layer, against the oracle.
Tolerances as for one layer: 1e-12 relative max-norm in FP64 and f32x2,
2e-5 in FP32 (1e-4 for the radiation case, see test_border_gpu).
"""
from __future__ import annotations

import numpy as np
import pytest

import cases
import oracle as O
from test_border_gpu import RAD_TOL, affine, run_radiation, run_table
from test_oracle_golden import layers_case

pytestmark = pytest.mark.gpu

TOL = {"f64": 1e-12, "f32x2": 1e-12, "f32": 2e-5}


@pytest.mark.parametrize("prec", ["f64", "f32x2", "f32"])
def test_dirichlet_two_layers_golden(gpu, prec):
    M = gpu
    d, g, S, T, nl = layers_case("heat_timelin_nl2")
    n = tuple(d["n"])
    cfg = M.make_cfg(n, tau=g.tau, precision=prec, heat=(1.0, 1.0, 0.0), n_layers=nl)
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_F_A, S)
        p.upload(M.FIELD_G_A, S)
        p.upload(M.FIELD_G_B, S)
        p.upload(M.FIELD_U, S * 1.0)
        p.step(T)
        u = p.download()
    assert cases.rel_err(u, d["final"]) <= TOL[prec]


@pytest.mark.parametrize("prec", ["f64", "f32x2", "f32"])
def test_neumann_three_layers_golden(gpu, prec):
    d, g, S, T, nl = layers_case("heat_neumann_nl3")
    n = tuple(d["n"])
    u = run_table(gpu, g, n, S * 1.0, T, 0, (S, 0, 1.0, 0.0), (S, 0, 1.0, 1.0),
                  (np.full(S.shape, -1.0), 0, 1.0, 1.0), prec, (1.0, 1.0, 0.0), n_layers=nl)
    assert cases.rel_err(u, d["final"]) <= TOL[prec]


@pytest.mark.parametrize("prec", ["f64", "f32x2", "f32"])
def test_radiation_two_layers_golden(gpu, prec):
    d, g, S, T, nl = layers_case("pennes_radiation_nl2")
    u = run_radiation(gpu, d, g, S, T, (0.5, 2.0), prec, n_layers=nl)
    assert cases.rel_err(u, d["final"]) <= RAD_TOL[prec]


@pytest.mark.parametrize("nl", [2, 3, 5])
@pytest.mark.parametrize("prec", ["f64", "f32x2", "f32"])
def test_dirichlet_layers_noisy(gpu, nl, prec):
    """66 x 40 x 35: with 2 layers the tile at x = 32 is inner, with 3 and 5
    it reaches into the border layer; every tile row and z-chunk edge meets
    the layer somewhere."""
    M = gpu
    n, T = (66, 40, 35), 30
    shape = (n[2], n[1], n[0])
    rng = np.random.default_rng(50 + nl)
    h2 = sum((m - 1) ** 2 for m in n)
    tau = 0.9 / (2.0 * h2)
    g = O.make_grid(n, tau=tau, n_layers=nl)
    u0 = rng.uniform(-1.0, 1.0, shape)
    fb = rng.uniform(-1.0, 1.0, shape)
    gb = rng.uniform(-1.0, 1.0, shape)
    ref = O.heat_dirichlet(g, u0, T, f_base=fb, f_a=1.0, f_b=0.5, g_base=gb, g_a=1.0, g_b=-2.0)
    fa, fbb = affine((fb, 0, 1.0, 0.5), shape)
    ga, gbb = affine((gb, 0, 1.0, -2.0), shape)
    cfg = M.make_cfg(n, tau=tau, precision=prec, heat=(1.0, 1.0, 0.0), n_layers=nl)
    for tile in range(1, 5):
        cfg.tile = tile
        with M.Plain(cfg) as p:
            p.upload(M.FIELD_F_A, fa)
            p.upload(M.FIELD_F_B, fbb)
            p.upload(M.FIELD_G_A, ga)
            p.upload(M.FIELD_G_B, gbb)
            p.upload(M.FIELD_U, u0)
            p.step(T)
            u = p.download()
        assert cases.rel_err(u, ref) <= TOL[prec], (nl, prec, tile)
