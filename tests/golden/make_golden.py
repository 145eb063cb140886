"""Generates the golden vectors in tests/golden/ by running the reference.

Each case runs one of the reference-driver programs in oracle/_ref/ -- the
reference's own Problem::iterateOverTime() and, where the reference has one,
its own system-test problem class, compiled from the untouched reference
headers by ``make -C oracle ref`` -- and stores its inputs and final iterate.

Run from the repository root (needs the reference checkout for the build):

    make -C oracle ref && python tests/golden/make_golden.py [--tissue | --tangent | --lame-first-order]

The .npz files are committed; the GPU machine never runs this script.
"""
from __future__ import annotations

import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import oracle as O  # noqa: E402

sys.path.insert(0, str(ROOT / "tests"))
import cases  # noqa: E402

OUT = Path(__file__).resolve().parent


def ijk(n):
    k, j, i = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    return i, j, k


def sine_noise(n, seed, amp=1e-3):
    """sin(pi x) sin(pi y) sin(pi z) on the unit cube plus seeded uniform
    noise in [-amp, amp] at inner nodes; border nodes 0."""
    g = O.make_grid(n)
    x, y, z = O.coords(g)
    u0 = np.broadcast_to(np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z),
                         (n[2], n[1], n[0])).copy()
    border = O.border_mask(g)
    if amp:
        u0 += np.random.default_rng(seed).uniform(-amp, amp, u0.shape) * (~border)
    u0[border] = 0.0
    return u0


def main():
    tmp = tempfile.mkdtemp()
    cases = {}

    # tests/system/HeatEqnFdmStencilWidthOne/TESTMATRIX_RUN_3D.sh.in: 32^3, 20 steps,
    # coordinates 0..1000.
    n, T = (32, 32, 32), 20
    r = O.run_ref("ref_stencil_width_one", n, T, tmp, last=(1000.0, 1000.0, 1000.0))
    cases["stencil_width_one"] = dict(n=n, nsteps=T, last=(1000.0,) * 3, t_end=1.0, final=r)

    # tests/system/HeatEqnFDM/Dirichlet/TimeLinSpaceLin/RUN_3D.sh.in: 8^3, 300 steps, t in [0,1].
    n, T = (8, 8, 8), 300
    r = O.run_ref("ref_heat_timelin", n, T, tmp)
    cases["heat_timelin"] = dict(n=n, nsteps=T, t_end=1.0, final=r)

    # tests/system/PennesBioheatEqnFDM/Dirichlet/TimeLinSpaceLin/RUN_3D.sh.in: 8^3, 300 steps.
    r = O.run_ref("ref_pennes_timelin", n, T, tmp)
    cases["pennes_timelin"] = dict(n=n, nsteps=T, t_end=1.0, final=r)

    # Flux-condition borders: tests/system/{HeatEqnFDM,PennesBioheatEqnFDM}/{Neumann,Cauchy}/
    # TimeLinSpaceLin/RUN_3D.sh.in (8^3, 300 steps, t in [0,1]) plus a non-cubic grid.
    for name in ("heat_neumann", "heat_cauchy", "pennes_neumann", "pennes_cauchy"):
        r = O.run_ref(f"ref_{name}", n, T, tmp)
        cases[name] = dict(n=n, nsteps=T, t_end=1.0, final=r)
    r = O.run_ref("ref_heat_neumann", (10, 8, 6), 320, tmp)
    cases["heat_neumann_10x8x6"] = dict(n=(10, 8, 6), nsteps=320, t_end=1.0, final=r)

    # Radiation border: tests/system/PennesBioheatEqnFDM/Radiation/TimeLinSpaceLin/RUN_3D.sh.in
    # (8^3, 50000 steps, t in [0,1]) plus a non-cubic grid.  The explicit u^4 flux bounds
    # the step: at a corner the linearised factor is 1 - tau * 8 u^3 * sum_p 1/h_p, which
    # must stay above -1 (u reaches 8; sum 1/h_p = 21 on both grids, so T > 43000).
    r = O.run_ref("ref_pennes_radiation", n, 50000, tmp)
    cases["pennes_radiation"] = dict(n=n, nsteps=50000, t_end=1.0, final=r)
    r = O.run_ref("ref_pennes_radiation", (10, 8, 6), 60000, tmp)
    cases["pennes_radiation_10x8x6"] = dict(n=(10, 8, 6), nsteps=60000, t_end=1.0, final=r)

    # nLayersAtBorder > 1 (src/ScaFES_Problem.hpp:3952-3971): the same system tests with
    # two or three border layers on a 12x10x9 grid (steps within the stability limits).
    nb = (12, 10, 9)
    for name, ref, T, nl in (("heat_timelin_nl2", "ref_heat_timelin", 800, 2),
                             ("heat_neumann_nl3", "ref_heat_neumann", 800, 3),
                             ("pennes_radiation_nl2", "ref_pennes_radiation", 60000, 2)):
        r = O.run_ref(ref, nb, T, tmp, n_layers=nl)
        cases[name] = dict(n=nb, nsteps=T, t_end=1.0, n_layers=nl, final=r)

    # tests/system/HeatEqnFdmStencilWidthVar/TESTMATRIX_RUN_3D.sh.in: 32^3, 20 steps.
    n, T = (32, 32, 32), 20
    r = O.run_ref("ref_stencil_width_var", n, T, tmp, nfields=3)
    cases["stencil_width_var"] = dict(n=n, nsteps=T, t_end=1.0, final=r)

    # Heat, sine mode + seeded noise, Dirichlet 0, tau = 0.9 of the stability limit.
    for name, n, T, seed in (("heat_noise_16", (16, 16, 16), 50, 2), ("heat_noise_odd", (17, 9, 5), 30, 3)):
        h2 = sum(1.0 / ((1.0 / (m - 1)) ** 2) for m in n)
        tau = 0.9 / (2.0 * h2)
        u0 = sine_noise(n, seed)
        r = O.run_ref("ref_heat_dirichlet", n, T, tmp, tau=tau, t_end=tau * T, inputs=u0)
        cases[name] = dict(n=n, nsteps=T, tau=tau, t_end=tau * T, u0=u0, final=r)

    # Variable-coefficient Pennes (MRI form), Dirichlet 37, seeded data.
    n, T = (12, 10, 9), 100
    rng = np.random.default_rng(8)
    shape = (n[2], n[1], n[0])
    u0 = 37.0 + rng.uniform(-1.0, 1.0, shape)
    q = rng.uniform(0.0, 10.0, shape)
    gb = np.full(shape, 37.0)
    params = np.array([1.0, 1.0, 0.5, 1.0, 1.0, 2e-3, 37.0])  # rho c k rho_b c_b omega T_b
    tau = 1e-4
    r = O.run_ref("ref_pennes_mri", n, T, tmp, tau=tau, t_end=tau * T,
                  inputs=np.concatenate([u0.ravel(), q.ravel(), gb.ravel()]), extra=params)
    cases["pennes_mri"] = dict(n=n, nsteps=T, tau=tau, t_end=tau * T, u0=u0, q=q, g=gb,
                               params=params, final=r)

    cases.update(tissue_cases(tmp))
    cases.update(tangent_cases(tmp))
    cases.update(lame_first_order_cases(tmp))
    save(cases)


def tangent_cases(tmp):
    """Directional derivatives of J = 1/2 ||u_T - target||^2 for the heat
    update with a zero Dirichlet border, taken through the reference's own
    updateInner<TT>/updateBorder<TT> with a dual number (ref_heat_tangent):
    dJ_k = <u_T - target, du_T along d_k>, the numbers the adjoint's
    <dJ/du0, d_k> must reproduce -- for directions over all nodes (dJ) and
    the same directions with a zero border (dJ_inner).  A border value of
    u0 enters only the first step: the Dirichlet border resets it."""
    n, T = (32, 32, 32), 60
    tau = 0.9 / (2.0 * sum((m - 1) ** 2 for m in n))
    u0, target, dirs = cases.tangent_inputs(n)
    # The four directions over all nodes, then the same with a zero border.
    border = O.border_mask(O.make_grid(n))
    inner_dirs = [np.where(border, 0.0, d) for d in dirs]
    r = O.run_ref("ref_heat_tangent", n, T, tmp, tau=tau, t_end=tau * T,
                  inputs=np.concatenate([u0.ravel()] + [d.ravel() for d in dirs + inner_dirs]),
                  extra=[2 * len(dirs)], nfields=1 + 2 * len(dirs))
    uT = r[0]
    dJ = np.array([float(np.sum((uT - target) * r[1 + k])) for k in range(2 * len(dirs))])
    return {"heat_tangent_32": dict(n=n, nsteps=T, tau=tau, t_end=tau * T, uT=uT, dJ=dJ[:len(dirs)],
                                    dJ_inner=dJ[len(dirs):])}


# The reference's tissue examples (examples/TumorHeatEqnFDM, examples/
# MRIDataPBHEqnFDM), compiled unmodified: per-node coefficients and the
# examples' own flux borders.
TUMOUR_PARAMS = dict(RHO=1040.0, C=3650.0, K=0.6, Q_BRAIN=25000.0, Q_TUMOR=60000.0, RHO_B=1052.0, C_PB=3800.0,
                     OMEGA_B_BRAIN=0.004, OMEGA_B_TUMOR=0.0007, T_I=37.0, H=10.0, T_INF=22.4, Q_BC=0.0,
                     DIAMETER=0.01, DEPTH=0.008, T_A=37.0)
TUMOUR_ORDER = ("RHO", "C", "K", "Q_BRAIN", "Q_TUMOR", "RHO_B", "C_PB", "OMEGA_B_BRAIN", "OMEGA_B_TUMOR", "T_I",
                "H", "T_INF", "Q_BC", "DIAMETER", "DEPTH", "T_A")
MRI_ORDER = ("H", "T_INF", "Q_BC", "Q_SKULL", "EPSILON", "T_INIT")


def mri_fields(n, seed):
    """Seeded tissue fields of the MRI example over the nodes (uniform per
    node in physiological ranges), in oracle.TISSUE_FIELDS order."""
    shape = (n[2], n[1], n[0])
    rng = np.random.default_rng(seed)
    ranges = {"rho": (1000, 1100), "c": (3500, 3800), "k": (0.4, 0.6), "rho_b": (1040, 1060),
              "c_b": (3700, 3900), "omega": (0.001, 0.005), "t_blood": (36.5, 37.5), "q": (1e4, 3e4)}
    return np.stack([rng.uniform(*ranges[k], shape) for k in O.TISSUE_FIELDS])


def tissue_cases(tmp):
    cases = {}
    # Tumour example on its domain (0.06 x 0.03 x 0.03 m, Parameters.ini.in values, a
    # hotter tumour), coarser grid, 200 steps of 5 s (below the stability limit).
    n, T, tau, last = (20, 12, 12), 200, 5.0, (0.06, 0.03, 0.03)
    P = TUMOUR_PARAMS
    r = O.run_ref("ref_tumor_example", n, T, tmp, tau=tau, t_end=tau * T, last=last, inputs=np.zeros(1),
                  extra=[P[k] for k in TUMOUR_ORDER])
    cases["tissue_tumour"] = dict(n=n, nsteps=T, tau=tau, t_end=tau * T, last=last,
                                  params=np.array([P[k] for k in TUMOUR_ORDER]), final=r)
    # MRI example with seeded coefficient fields: closed skull (linear borders) and an
    # open-skull patch on the z-max face (convection + radiation).
    n, T, tau, last = (14, 12, 10), 100, 5.0, (0.05, 0.04, 0.03)
    par = dict(H=10.0, T_INF=22.0, Q_BC=5.0, Q_SKULL=-3.0, EPSILON=0.98, T_INIT=37.0)
    fields = mri_fields(n, 31)
    for name, patch in (("tissue_mri_closed", False), ("tissue_mri_open", True)):
        surface = np.zeros((n[2], n[1], n[0]))
        if patch:
            surface[-1, 3:9, 4:10] = 1.0
        r = O.run_ref("ref_mri_example", n, T, tmp, tau=tau, t_end=tau * T, last=last,
                      inputs=np.concatenate([fields, surface[None]]), extra=[par[k] for k in MRI_ORDER])
        cases[name] = dict(n=n, nsteps=T, tau=tau, t_end=tau * T, last=last, fields=fields, surface=surface,
                           params=np.array([par[k] for k in MRI_ORDER]), final=r)
    return cases


def lame_first_order_cases(tmp):
    """The reference's first-order Lame-Navier example (examples/
    LameNavierEqnFDMFirstOrder), compiled unmodified: six unknown fields
    coupled through its updateInner/updateBorder, known fields zero, its own
    initial state (V3 = omega); a time step small enough for the example's
    stiff constants (lambda ~ 1.7e9)."""
    cases = {}
    for name, n, T, tau in (("lame_first_order", (12, 10, 9), 40, 1e-10),
                            ("lame_first_order_b", (17, 9, 13), 25, 5e-11)):
        r = O.run_ref("ref_lame_first_order", n, T, tmp, tau=tau, t_end=tau * T, inputs=None, nfields=6)
        cases[name] = dict(n=n, nsteps=T, tau=tau, t_end=tau * T, final=r)
    return cases


def save(cases):
    for name, c in cases.items():
        arrays = {k: np.asarray(v) for k, v in c.items()}
        np.savez_compressed(OUT / f"{name}.npz", **arrays)
        print(f"{name}: {OUT / (name + '.npz')}")


if __name__ == "__main__":
    if sys.argv[1:] == ["--tissue"]:   # only the tissue-example cases
        save(tissue_cases(tempfile.mkdtemp()))
    elif sys.argv[1:] == ["--tangent"]:  # only the dual-number gradient case
        save(tangent_cases(tempfile.mkdtemp()))
    elif sys.argv[1:] == ["--lame-first-order"]:  # only the multi-unknown example
        save(lame_first_order_cases(tempfile.mkdtemp()))
    else:
        main()
