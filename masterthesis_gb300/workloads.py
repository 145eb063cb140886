"""Seeded synthetic inputs of the benchmark workloads.

The reference measures wall time on synthetic problems only; these
generators reproduce the shapes, sizes and value distributions of the
workloads the engine is measured on:

* ``heat_sine_noise``: sin(pi x) sin(pi y) sin(pi z) on the unit cube plus
  seeded uniform noise at inner nodes, border 0 (the plain heat workloads);
* ``pennes_ensemble``: independent Pennes bioheat instances with seeded
  grid sizes, conductivity, perfusion and a Gaussian heat source each
  (the batched ensemble workload);
* ``tissue_fields_slab`` / ``tissue_device_form``: Pennes bioheat with every
  coefficient a field over the nodes and the flux borders of the reference's
  tissue examples (the variable-coefficient workload).
"""
from __future__ import annotations

import numpy as np


def heat_tau(n, alpha: float = 1.0, safety: float = 0.9) -> float:
    """``safety`` times the explicit-Euler stability limit
    1 / (2 alpha sum_p 1/h_p^2) on the unit cube."""
    return safety / (2.0 * alpha * sum((m - 1) ** 2 for m in n))


def heat_sine_noise(n, seed: int = 2, amp: float = 1e-3, out: np.ndarray | None = None) -> np.ndarray:
    """Initial iterate of the plain heat workloads, shape (nz, ny, nx),
    built plane by plane (so 512^3 needs no temporaries of full size)."""
    nx, ny, nz = n
    sx = np.sin(np.pi * np.arange(nx) / (nx - 1))
    sy = np.sin(np.pi * np.arange(ny) / (ny - 1))
    sz = np.sin(np.pi * np.arange(nz) / (nz - 1))
    u = np.empty((nz, ny, nx)) if out is None else out
    rng = np.random.default_rng(seed)
    for k in range(nz):
        plane = sz[k] * (sy[:, None] * sx[None, :])
        if amp:
            plane = plane + rng.uniform(-amp, amp, (ny, nx))
        if k == 0 or k == nz - 1:
            plane[:] = 0.0
        else:
            plane[0, :] = plane[-1, :] = 0.0
            plane[:, 0] = plane[:, -1] = 0.0
        u[k] = plane
    return u


T_ARTERIAL = 37.0


def pennes_ensemble(n_inst: int = 256, seed: int = 8, sizes=tuple(range(32, 161, 16)),
                    safety: float = 0.9):
    """Pennes bioheat ensemble (rho c = rho_b c_b = 1, arterial and initial
    temperature 37, Dirichlet 37).  Per instance: grid size per axis drawn
    from ``sizes``, k ~ U[0.4, 0.6], w_b ~ U[0.5, 5]e-3, and a Gaussian heat
    source Q = A exp(-|x - c|^2 / (2 s^2)) with c ~ U[0.3, 0.7]^3,
    s ~ U[0.05, 0.15], A ~ U[1, 10].  The time step is ``safety`` times the
    stability limit of that instance.  Returns a list of dicts with keys
    n (nx, ny, nz), k, w_b, tau, q (array (nz, ny, nx))."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n_inst):
        n = tuple(int(v) for v in rng.choice(np.asarray(sizes), size=3))
        k = float(rng.uniform(0.4, 0.6))
        w_b = float(rng.uniform(0.5, 5.0) * 1e-3)
        c = rng.uniform(0.3, 0.7, 3)
        s = float(rng.uniform(0.05, 0.15))
        amp = float(rng.uniform(1.0, 10.0))
        x = np.arange(n[0]) / (n[0] - 1)
        y = np.arange(n[1]) / (n[1] - 1)
        z = np.arange(n[2]) / (n[2] - 1)
        r2 = ((x[None, None, :] - c[0]) ** 2 + (y[None, :, None] - c[1]) ** 2 + (z[:, None, None] - c[2]) ** 2)
        q = amp * np.exp(-r2 / (2.0 * s * s))
        tau = safety / (2.0 * k * sum((m - 1) ** 2 for m in n) + w_b)
        out.append({"n": n, "k": k, "w_b": w_b, "tau": tau, "q": q})
    return out


def pennes_batch_instance(spec: dict):
    """The C ABI instance of one ensemble member (source F = w_b T_a + Q)."""
    from masterthesis_gb300 import batch_instance
    return batch_instance(spec["n"], spec["tau"], coeff_a=spec["k"], rho_c=1.0, perf=spec["w_b"],
                          g_value=T_ARTERIAL)


def pennes_source(spec: dict) -> np.ndarray:
    return spec["w_b"] * T_ARTERIAL + spec["q"]


def gaussian_bump_displacement(n, seed: int = 3):
    """Lame-Navier initial displacement: a seeded Gaussian bump per
    component (centre c ~ U[0.35, 0.65]^3, width s ~ U[0.05, 0.1],
    amplitude ~ U[-1, 1] per component), zero on the border.  Shape
    (3, nz, ny, nx)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.35, 0.65, 3)
    s = float(rng.uniform(0.05, 0.1))
    amp = rng.uniform(-1.0, 1.0, 3)
    x = np.arange(n[0]) / (n[0] - 1)
    y = np.arange(n[1]) / (n[1] - 1)
    z = np.arange(n[2]) / (n[2] - 1)
    r2 = (x[None, None, :] - c[0]) ** 2 + (y[None, :, None] - c[1]) ** 2 + (z[:, None, None] - c[2]) ** 2
    bump = np.exp(-r2 / (2.0 * s * s))
    u = np.stack([a * bump for a in amp])
    u[:, 0, :, :] = u[:, -1, :, :] = 0.0
    u[:, :, 0, :] = u[:, :, -1, :] = 0.0
    u[:, :, :, 0] = u[:, :, :, -1] = 0.0
    return u


def lame_tau(n, lam=1.0, mu=0.5, rho=1.0, safety: float = 0.5) -> float:
    """A stable leapfrog step for the Lame-Navier scheme: ``safety`` times
    h / (c_p sqrt(3)) with the pressure-wave speed c_p = sqrt((lam+2mu)/rho)."""
    h = 1.0 / (max(n) - 1)
    return safety * h / (np.sqrt((lam + 2.0 * mu) / rho) * np.sqrt(3.0))


def yee_setup(n, seed: int = 4, courant: float = 0.5):
    """Yee workload: tau = courant * h / sqrt(3) (eps = mu = 1) and a seeded
    point dipole (Ez soft source) near the centre; source parameters
    (amp, t0, w, freq) of a Gaussian-modulated sine a few periods long."""
    rng = np.random.default_rng(seed)
    h = 1.0 / (n[0] - 1)
    tau = courant * h / np.sqrt(3.0)
    src = tuple(int(v) for v in (np.array(n) // 2 + rng.integers(-2, 3, 3)))
    freq = 4.0
    w = 1.0 / freq
    return tau, src, (1.0, 2.0 * w, w, freq)


def yee_linear_rules(ch: float) -> dict:
    """The Yee cavity without a source (the staggering of the fused Yee
    kernels, ch = tau / h) as rules of the linear multi-field kernel
    (scafes_lin_*): phase 1 the H half step, phase 2 the E step on its
    result; fields Ex Ey Ez Hx Hy Hz; {(phase, field, class): terms} with
    terms (src, dx, dy, dz, w).  A node of class c has no +p neighbour when
    bit 2p+1 is set and is inner along p when neither bit 2p nor 2p+1 is."""
    unit = ((1, 0, 0), (0, 1, 0), (0, 0, 1))
    rules = {}
    for cls in range(64):
        has_up = [not (cls >> (2 * p + 1)) & 1 for p in range(3)]
        inner = [has_up[p] and not (cls >> (2 * p)) & 1 for p in range(3)]
        for c in range(3):
            a, b = (c + 1) % 3, (c + 2) % 3
            ident_e, ident_h = [(c, 0, 0, 0, 1.0)], [(3 + c, 0, 0, 0, 1.0)]
            # H_c -= ch ((E_b(+a) - E_b) - (E_a(+b) - E_a))
            rules[(1, 3 + c, cls)] = (ident_h + [(b, *unit[a], -ch), (b, 0, 0, 0, ch), (a, *unit[b], ch),
                                                 (a, 0, 0, 0, -ch)]) if has_up[a] and has_up[b] else ident_h
            rules[(1, c, cls)] = ident_e
            # E_c += ch ((H_b - H_b(-a)) - (H_a - H_a(-b)))
            down_a = tuple(-v for v in unit[a])
            down_b = tuple(-v for v in unit[b])
            rules[(2, c, cls)] = (ident_e + [(3 + b, 0, 0, 0, ch), (3 + b, *down_a, -ch), (3 + a, 0, 0, 0, -ch),
                                             (3 + a, *down_b, ch)]) if has_up[c] and inner[a] and inner[b] else ident_e
            rules[(2, 3 + c, cls)] = ident_h
    return rules


# ---- tissue workloads (coefficients per node) ----------------------------------

TISSUE_FIELDS = ("rho", "c", "k", "rho_b", "c_b", "omega", "t_blood", "q")
TISSUE_RANGES = {"rho": (1000.0, 1100.0), "c": (3500.0, 3800.0), "k": (0.4, 0.6), "rho_b": (1040.0, 1060.0),
                 "c_b": (3700.0, 3900.0), "omega": (0.001, 0.005), "t_blood": (36.5, 37.5), "q": (1e4, 3e4)}


def tissue_fields_slab(n, z0: int, z1: int, seed: int) -> dict:
    """Seeded tissue coefficients of planes z0..z1-1 of an nx x ny x nz grid
    (the known fields of the MRI-data Pennes example: density, heat capacity,
    conductivity, blood density and heat capacity, perfusion, blood
    temperature, metabolic heat), uniform per node in physiological ranges;
    each plane has its own stream, so slabs of any size give the same
    field."""
    nx, ny = n[0], n[1]
    out = {k: np.empty((z1 - z0, ny, nx)) for k in TISSUE_FIELDS}
    for z in range(z0, z1):
        rng = np.random.default_rng((seed, z))
        for k in TISSUE_FIELDS:
            out[k][z - z0] = rng.uniform(*TISSUE_RANGES[k], (ny, nx))
    return out


def tissue_device_form(n, h, tau, fields: dict, z0: int = 0, flux: dict | None = None):
    """The device form of the tissue examples' update on planes z0.. of the
    grid (the form the drop-in Problem records from their callbacks):

      inner node:  C0 = 1 - 2 sum_p s_p - tau P,  CA = tau a,
                   F  = tau P T_b + tau q/(rho c)   (source weight cf = 1),
      with a = k/(rho c), s_p = tau a/h_p^2, P = rho_b c_b omega/(rho c), and
      the axis factors cp = 1/h_p^2;
      border node (flux border, when `flux` is given): the examples' bracket
      per axis -- the missing neighbour replaced by the inner one plus a
      flux term: Neumann q_bc at the min faces and the x, y max faces, at the
      z max face Neumann q_skull (zmax_kind 0) or Cauchy h_conv, t_amb
      (zmax_kind 1) -- as one rule (cu, cn[6], cst) per border node, the
      border nodes of the slab in Fortran order.

    fields maps TISSUE_FIELDS to arrays (or scalars) over the slab's planes.
    Returns dict C0, CA, F (slab arrays), cp, rules ((m, 8) or None)."""
    nzs = next(np.shape(v)[0] for v in fields.values() if np.ndim(v) == 3)
    shape = (nzs, n[1], n[0])
    f = {k: np.broadcast_to(np.asarray(fields[k], dtype=np.float64), shape) for k in TISSUE_FIELDS}
    rho_c = f["rho"] * f["c"]
    a = f["k"] / rho_c
    P = (f["rho_b"] * f["c_b"]) / rho_c * f["omega"]
    s = [tau * a / (hp * hp) for hp in h]
    out = {"C0": 1.0 - 2.0 * (s[0] + s[1] + s[2]) - tau * P, "CA": tau * a,
           "F": tau * P * f["t_blood"] + tau * (1.0 / rho_c) * f["q"], "cp": [1.0 / (hp * hp) for hp in h],
           "rules": None}
    if flux is None:
        return out
    kz, ky, kx = np.meshgrid(np.arange(z0, z0 + nzs), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    pos = (kx, ky, kz)
    border = (kx == 0) | (kx == n[0] - 1) | (ky == 0) | (ky == n[1] - 1) | (kz == 0) | (kz == n[2] - 1)
    cu = 1.0 - tau * P
    cst = out["F"].copy()
    cn = np.zeros((6,) + shape)
    for p in range(3):
        at_min = pos[p] == 0
        at_max = pos[p] == n[p] - 1
        fl = s[p] * (2.0 * h[p] / f["k"])
        cu = cu - 2.0 * s[p]
        cn[2 * p] = np.where(at_min, 0.0, np.where(at_max, 2.0 * s[p], s[p]))
        cn[2 * p + 1] = np.where(at_max, 0.0, np.where(at_min, 2.0 * s[p], s[p]))
        if p == 2 and flux.get("zmax_kind", 0) == 1:
            cu = cu - np.where(at_max, fl * flux["h_conv"], 0.0)
            cst = cst + np.where(at_max, fl * flux["h_conv"] * flux["t_amb"], 0.0)
        else:
            q_max = flux.get("q_skull", 0.0) if p == 2 else flux.get("q_bc", 0.0)
            cst = cst + np.where(at_max, fl * q_max, 0.0)
        cst = cst + np.where(at_min, fl * flux.get("q_bc", 0.0), 0.0)
    sel = border.ravel()
    rules = np.empty((int(sel.sum()), 8))
    rules[:, 0] = np.broadcast_to(cu, shape).ravel()[sel]
    for d in range(6):
        rules[:, 1 + d] = cn[d].ravel()[sel]
    rules[:, 7] = cst.ravel()[sel]
    out["rules"] = rules
    return out


def tissue_tau(n, last, safety: float = 0.9) -> float:
    """`safety` times the stability limit of the tissue update for the
    largest diffusivity the seeded fields reach (k/(rho c) <= 0.6/3.5e6)."""
    a_max = TISSUE_RANGES["k"][1] / (TISSUE_RANGES["rho"][0] * TISSUE_RANGES["c"][0])
    return safety / (2.0 * a_max * sum(((m - 1) / L) ** 2 for m, L in zip(n, last)))
