"""Variable-coefficient update and per-node border rules (C ABI, CUDA).

The reference's tissue examples -- TumorHeatEqnFDM (perfusion and heat
source change inside a tumour sphere, Cauchy z-max face) and
MRIDataPBHEqnFDM (every coefficient a field over the nodes; closed skull:
Neumann borders) -- run through the coefficient slots C0/CA, the source
F_A and SCAFES_BORDER_NODES, against the golden vectors of the reference's
own classes (tests/golden/tissue_*.npz).  Further cases: the MRI form with a
Dirichlet border against the oracle on ragged grids and every tile variant,
plain FP32, and the refusals.  Tolerances: relative max-norm 1e-12 (FP64),
1e-5 (FP32: one FP32 rounding per step on temperatures near 37).
"""
from __future__ import annotations

import numpy as np
import pytest

import cases
import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["tissue_tumour", "tissue_mri_closed"])
@pytest.mark.parametrize("tile", [0, 1, 2, 3, 4])
def test_tissue_examples_match_reference(gpu, name, tile):
    d, g, fields, kw, u0 = cases.tissue_case(name)
    dev = cases.tissue_device_inputs(g, fields, kw)
    u = cases.run_tissue(kw, g, dev, u0, int(d["nsteps"]), tile=tile)
    assert cases.rel_err(u, d["final"]) <= 1e-12


@pytest.mark.parametrize("name", ["tissue_tumour", "tissue_mri_closed"])
def test_tissue_examples_f32(gpu, name):
    d, g, fields, kw, u0 = cases.tissue_case(name)
    dev = cases.tissue_device_inputs(g, fields, kw)
    u = cases.run_tissue(kw, g, dev, u0, int(d["nsteps"]), precision="f32")
    assert cases.rel_err(u, d["final"]) <= 1e-5


@pytest.mark.parametrize("n", [(37, 19, 23), (64, 40, 9), (33, 65, 17)])
@pytest.mark.parametrize("tile", [1, 2, 3, 4])
def test_mri_form_dirichlet_matches_oracle(gpu, n, tile):
    """Ragged grids (tiles cut in x, y and z) with a Dirichlet border from a
    field: the variable-coefficient sweep against the oracle's restatement
    of the MRI example's updateInner."""
    M = gpu
    shape = (n[2], n[1], n[0])
    rng = np.random.default_rng(sum(n) + tile)
    last = (0.05, 0.04, 0.03)
    ranges = {"rho": (1000, 1100), "c": (3500, 3800), "k": (0.4, 0.6), "rho_b": (1040, 1060),
              "c_b": (3700, 3900), "omega": (0.001, 0.005), "t_blood": (36.5, 37.5), "q": (1e4, 3e4)}
    fields = {k: rng.uniform(*v, shape) for k, v in ranges.items()}
    hmin = min(last[p] / (n[p] - 1) for p in range(3))
    tau = 0.45 * 1000 * 3500 / 0.6 * hmin * hmin / 3.0
    g = O.make_grid(n, last=last, tau=tau)
    gb = rng.uniform(36.0, 38.0, shape)
    u0 = rng.uniform(36.0, 38.0, shape)
    T = 30
    ref = O.pennes_tissue(g, u0, T, fields, g_bdry=gb)
    dev = cases.tissue_device_inputs(g, fields, {})
    u = cases.run_tissue({}, g, dev, u0, T, border="dirichlet", g_bdry=gb, tile=tile)
    assert cases.rel_err(u, ref) <= 1e-12


def test_variable_coefficient_refusals(gpu):
    M = gpu
    n = (12, 10, 9)
    shape = (n[2], n[1], n[0])
    ones = np.ones(shape)
    # F32X2 is not a variable-coefficient precision.
    cfg = M.make_cfg(n, tau=1e-4, precision="f32x2", c0=1.0, cp=(1.0, 1.0, 1.0), cf=1.0)
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_C0, ones)
        p.upload(M.FIELD_CA, 0.01 * ones)
        p.upload(M.FIELD_U, ones)
        with pytest.raises(M.ScafesError) as e:
            p.step(1)
        assert e.value.code == -4
    cfg = M.make_cfg(n, tau=1e-4, c0=1.0, cp=(1.0, 1.0, 1.0), cf=1.0)
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_C0, ones)  # CA missing
        p.upload(M.FIELD_U, ones)
        with pytest.raises(M.ScafesError) as e:
            p.step(1)
        assert e.value.code == -3
    # Per-node border: the rules are missing, the count is wrong, a rule
    # weights a neighbour outside the grid; F32X2 is refused at create.
    cfg = M.make_cfg(n, tau=1e-4, c0=1.0, cp=(1.0, 1.0, 1.0), cf=1.0, border=M.BORDER_NODES)
    m = M.border_node_count(cfg)
    assert m == 12 * 10 * 9 - 10 * 8 * 7
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_C0, ones)
        p.upload(M.FIELD_CA, 0.01 * ones)
        p.upload(M.FIELD_U, ones)
        with pytest.raises(M.ScafesError) as e:
            p.step(1)
        assert e.value.code == -3
        with pytest.raises(M.ScafesError) as e:
            p.set_border_node_rules(np.zeros((m - 1, 8)))
        assert e.value.code == -1
        bad = np.zeros((m, 8))
        bad[0, 1] = 1.0  # node (0,0,0): weight on its x- neighbour
        with pytest.raises(M.ScafesError) as e:
            p.set_border_node_rules(bad)
        assert e.value.code == -1
    with pytest.raises(M.ScafesError) as e:
        M.Plain(M.make_cfg(n, tau=1e-4, precision="f32x2", c0=1.0, cp=(1.0, 1.0, 1.0), border=M.BORDER_NODES))
    assert e.value.code == -4
