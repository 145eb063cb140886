"""Inputs of the golden cases for the CUDA path (test infrastructure).

Each builder returns the scafes_cfg arguments and the host arrays to upload
for one golden case of tests/golden/, with the known fields written in the
affine-in-time form the C ABI takes (K(t) = K_A + time(t) * K_B).
"""
from __future__ import annotations

import numpy as np

import masterthesis_gb300 as M
import oracle as O
from conftest import load_golden


def unit_grid(n, last=(1.0, 1.0, 1.0), tau=0.0):
    return O.make_grid(n, last=last, tau=tau)


def lin_s(g):
    """1 + x + y + z in the reference's evaluation order
    (tests/system/HeatEqnFDM/Dirichlet/TimeLinSpaceLin/TimeLinSpaceLin.hpp:82-85)."""
    x, y, z = O.coords(g)
    return np.broadcast_to(((1.0 + x) + y) + z, (g.n[2], g.n[1], g.n[0])).copy()


def heat_noise(name, precision):
    d = load_golden(name)
    n = tuple(int(v) for v in d["n"])
    tau = float(d["tau"])
    cfg = M.make_cfg(n, tau=tau, precision=precision, heat=(1.0, 1.0, 0.0))
    return d, cfg, {M.FIELD_U: d["u0"]}


def heat_timelin(precision):
    d = load_golden("heat_timelin")
    n = tuple(int(v) for v in d["n"])
    T = int(d["nsteps"])
    tau = float(d["t_end"]) / T
    g = unit_grid(n, tau=tau)
    S = lin_s(g)
    cfg = M.make_cfg(n, tau=tau, precision=precision, heat=(1.0, 1.0, 0.0))
    fields = {M.FIELD_U: S, M.FIELD_F_A: S, M.FIELD_G_A: S, M.FIELD_G_B: S,
              M.FIELD_E_A: S, M.FIELD_E_B: S}
    return d, cfg, fields


def pennes_timelin(precision):
    """Pennes system test: perfusion rho_b c_b W/(rho c) = 1 and
    f(t) = S + S (1 + t) (PennesBioheatEqnFDM/Dirichlet/TimeLinSpaceLin)."""
    d = load_golden("pennes_timelin")
    n = tuple(int(v) for v in d["n"])
    T = int(d["nsteps"])
    tau = float(d["t_end"]) / T
    g = unit_grid(n, tau=tau)
    S = lin_s(g)
    cfg = M.make_cfg(n, tau=tau, precision=precision, heat=(1.0, 1.0, 1.0))
    fields = {M.FIELD_U: S, M.FIELD_F_A: 2.0 * S, M.FIELD_F_B: S, M.FIELD_G_A: S, M.FIELD_G_B: S,
              M.FIELD_E_A: S, M.FIELD_E_B: S}
    return d, cfg, fields


def stencil_width_one(precision):
    d = load_golden("stencil_width_one")
    n = tuple(int(v) for v in d["n"])
    k, j, i = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    c = 2.0 / 7.0
    cfg = M.make_cfg(n, last=tuple(float(v) for v in d["last"]), tau=1.0 / int(d["nsteps"]),
                     precision=precision, border=M.BORDER_MIRROR_POW2, c0=c, cp=(c, c, c), cf=0.0)
    return d, cfg, {M.FIELD_U: (i + j + k).astype(np.float64)}


def pennes_mri(precision):
    """MRI-form Pennes with scalar coefficients as a 7-point star:
    c_p = tau k/(rho c)/h_p^2, c0 = 1 - 2 sum c_p - tau (rho_b c_b/(rho c)) omega,
    cf = tau/(rho c), F = q + rho_b c_b omega T_b."""
    d = load_golden("pennes_mri")
    n = tuple(int(v) for v in d["n"])
    tau = float(d["tau"])
    rho, c, k, rho_b, c_b, omega, t_b = (float(v) for v in d["params"])
    cfg = M.make_cfg(n, tau=tau, precision=precision, heat=(k / (rho * c), rho * c,
                                                           (rho_b * c_b) / (rho * c) * omega))
    fields = {M.FIELD_U: d["u0"], M.FIELD_F_A: d["q"] + rho_b * c_b * omega * t_b,
              M.FIELD_G_A: d["g"]}
    return d, cfg, fields


def run(cfg, fields, nsteps):
    with M.Plain(cfg) as p:
        for f, a in fields.items():
            if f != M.FIELD_U:
                p.upload(f, a)
        p.upload(M.FIELD_U, fields[M.FIELD_U])
        p.step(nsteps)
        return p.download()


def rel_err(a, ref):
    return float(np.max(np.abs(a - ref)) / max(np.max(np.abs(ref)), 1e-300))


# ---- the reference's tissue examples (tests/golden/tissue_*.npz) -------------

TUMOUR_ORDER = ("RHO", "C", "K", "Q_BRAIN", "Q_TUMOR", "RHO_B", "C_PB", "OMEGA_B_BRAIN", "OMEGA_B_TUMOR", "T_I",
                "H", "T_INF", "Q_BC", "DIAMETER", "DEPTH", "T_A")
MRI_ORDER = ("H", "T_INF", "Q_BC", "Q_SKULL", "EPSILON", "T_INIT")


def tissue_case(name):
    """(golden dict, oracle grid, tissue fields, border keywords of
    oracle.pennes_tissue, initial iterate) of one tissue golden case."""
    d = load_golden(name)
    n = tuple(int(v) for v in d["n"])
    g = O.make_grid(n, last=tuple(d["last"]), tau=float(d["tau"]))
    shape = (n[2], n[1], n[0])
    if name == "tissue_tumour":
        P = dict(zip(TUMOUR_ORDER, d["params"]))
        fields = O.tumour_fields(g, P)
        kw = dict(zmax_kind=1, q_bc=P["Q_BC"], h_conv=P["H"], t_amb=P["T_INF"])
        u0 = np.full(shape, P["T_I"])
    else:
        P = dict(zip(MRI_ORDER, d["params"]))
        fields = dict(zip(O.TISSUE_FIELDS, d["fields"]))
        kw = dict(surface=d["surface"], zmax_kind=0, q_bc=P["Q_BC"], q_skull=P["Q_SKULL"], h_conv=P["H"],
                  t_amb=P["T_INF"], epsilon=P["EPSILON"])
        u0 = np.full(shape, P["T_INIT"])
    return d, g, fields, kw, u0


def tissue_device_inputs(g, fields, kw):
    """The device form of the tissue examples' update on grid g
    (workloads.tissue_device_form on the whole grid; kw: the border keywords
    of oracle.pennes_tissue, empty for a Dirichlet border)."""
    from masterthesis_gb300 import workloads as W
    n = (g.n[0], g.n[1], g.n[2])
    shape = (n[2], n[1], n[0])
    full = {k: np.broadcast_to(np.asarray(v, dtype=np.float64), shape) for k, v in fields.items()}
    flux = None if not kw else {k: kw[k] for k in ("zmax_kind", "q_bc", "q_skull", "h_conv", "t_amb") if k in kw}
    d = W.tissue_device_form(n, [g.h[0], g.h[1], g.h[2]], g.tau, full, 0, flux)
    return {"C0": np.ascontiguousarray(d["C0"]), "CA": np.ascontiguousarray(d["CA"]),
            "F": np.ascontiguousarray(d["F"]), "cp": d["cp"], "rules": d["rules"]}


def run_tissue(cfg_kw, g, dev, u0, nsteps, border="nodes", g_bdry=None, tile=0, precision="f64"):
    """Runs the tissue update through the C ABI: coefficient slots, source,
    and the per-node border rules (or a Dirichlet border from g_bdry)."""
    n = (g.n[0], g.n[1], g.n[2])
    cfg = M.make_cfg(n, first=tuple(g.first), last=tuple(g.last), tau=g.tau, precision=precision,
                     border=M.BORDER_NODES if border == "nodes" else M.BORDER_DIRICHLET,
                     c0=0.0, cp=dev["cp"], cf=1.0, tile=tile)
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_C0, dev["C0"])
        p.upload(M.FIELD_CA, dev["CA"])
        p.upload(M.FIELD_F_A, dev["F"])
        if border == "nodes":
            p.set_border_node_rules(dev["rules"])
        else:
            p.upload(M.FIELD_G_A, g_bdry)
        p.upload(M.FIELD_U, u0)
        p.step(nsteps)
        return p.download()


def tangent_inputs(n):
    """Seeded inputs of the gradient golden case (tests/golden/
    heat_tangent_32.npz): u0 uniform in [-1, 1] with a zero border (seed
    41), the target (seed 42) and four directions over all nodes (seeds
    43..46)."""
    shape = (n[2], n[1], n[0])
    g = O.make_grid(n)
    u0 = np.random.default_rng(41).uniform(-1.0, 1.0, shape)
    u0[O.border_mask(g)] = 0.0
    target = np.random.default_rng(42).uniform(-1.0, 1.0, shape)
    dirs = [np.random.default_rng(43 + k).uniform(-1.0, 1.0, shape) for k in range(4)]
    return u0, target, dirs


def yee_lin_rules(ch):
    """The plain Yee cavity (oracle/scafes_oracle.c orc_yee without its
    source) as rules of the linear multi-field kernel: phase 1 the H half
    step, phase 2 the E step on its result; fields Ex Ey Ez Hx Hy Hz.
    Returns {(phase, field, cls): terms}; a node class lacks the +p
    neighbour when bit 2p+1 is set and is not inner in p when bit 2p or
    2p+1 is set."""
    rules = {}
    e = [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
    for cls in range(64):
        up = [not (cls >> (2 * p + 1)) & 1 for p in range(3)]
        inner = [not (cls >> (2 * p)) & 1 and up[p] for p in range(3)]
        for c in range(3):
            a, b = (c + 1) % 3, (c + 2) % 3  # H_c from E_b along a and E_a along b
            if up[a] and up[b]:
                rules[(1, 3 + c, cls)] = [(3 + c, 0, 0, 0, 1.0), (b, *e[a], -ch), (b, 0, 0, 0, ch),
                                          (a, *e[b], ch), (a, 0, 0, 0, -ch)]
            else:
                rules[(1, 3 + c, cls)] = [(3 + c, 0, 0, 0, 1.0)]
            rules[(1, c, cls)] = [(c, 0, 0, 0, 1.0)]
            ma = tuple(-v for v in e[a])
            mb = tuple(-v for v in e[b])
            if up[c] and inner[a] and inner[b]:
                rules[(2, c, cls)] = [(c, 0, 0, 0, 1.0), (3 + b, 0, 0, 0, ch), (3 + b, *ma, -ch),
                                      (3 + a, 0, 0, 0, -ch), (3 + a, *mb, ch)]
            else:
                rules[(2, c, cls)] = [(c, 0, 0, 0, 1.0)]
            rules[(2, 3 + c, cls)] = [(3 + c, 0, 0, 0, 1.0)]
    return rules

