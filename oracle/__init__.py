"""CPU oracle for the ScaFES explicit update path -- TEST INFRASTRUCTURE ONLY.

Python access (ctypes) to ``liboracle_scafes.so``, the plain-C restatement of
the reference's update sweeps in ``scafes_oracle.c``, plus helpers that run the
reference-driver programs of ``oracle/_ref`` (built from the untouched
reference headers by ``make -C oracle ref``).  Only ``tests/``, the smoke
check and the CPU-baseline leg of ``bench.py`` import this package, as the
checker.  The product library never uses it.

Field arrays are float64 numpy arrays of shape (nz, ny, nx) in C order, which
is the reference's Fortran node order (x fastest) in memory.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle_scafes.so"
REF_DIR = HERE / "_ref"


def build(force: bool = False) -> Path:
    """Compile liboracle_scafes.so (gcc + OpenMP)."""
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < (HERE / "scafes_oracle.c").stat().st_mtime:
        subprocess.run(["make", "-C", str(HERE), "liboracle_scafes.so"], check=True,
                       capture_output=True)
    return LIB_PATH


def reference_dir() -> str | None:
    """The reference checkout, from the SCAFES_REFERENCE_DIR environment
    variable (default: a ``reference`` directory beside this repository's
    parent); None where it is absent."""
    cand = os.environ.get("SCAFES_REFERENCE_DIR") or str(HERE.parents[1] / "reference")
    return cand if Path(cand, "src", "ScaFES_Problem.hpp").exists() else None


def build_ref(reference: str | None = None) -> bool:
    """Compile the reference-driver programs into oracle/_ref (only where the
    reference checkout exists)."""
    reference = reference or reference_dir()
    if reference is None or not Path(reference, "src", "ScaFES_Problem.hpp").exists():
        return False
    subprocess.run(["make", "-C", str(HERE), "-j8", "ref", f"REF={reference}"], check=True,
                   capture_output=True)
    return True


class Grid(C.Structure):
    _fields_ = [("dim", C.c_int), ("n", C.c_int * 3), ("first", C.c_double * 3),
                ("last", C.c_double * 3), ("h", C.c_double * 3), ("tau", C.c_double),
                ("t_start", C.c_double), ("n_layers", C.c_int)]


class Tissue(C.Structure):
    _fields_ = [(f, C.POINTER(C.c_double)) for f in ("rho", "c", "k", "rho_b", "c_b", "omega", "t_blood", "q",
                                                      "surface")] + \
               [("zmax_kind", C.c_int)] + [(f, C.c_double) for f in ("q_bc", "q_skull", "h_conv", "t_amb",
                                                                     "epsilon", "sigma")] + \
               [("border", C.c_int), ("g_bdry", C.POINTER(C.c_double))]


class Known(C.Structure):
    _fields_ = [("base", C.POINTER(C.c_double)), ("form", C.c_int), ("a", C.c_double),
                ("b", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        dp = C.POINTER(C.c_double)
        L.orc_grid_init.argtypes = [C.POINTER(Grid), C.c_int, C.POINTER(C.c_int), dp, dp,
                                    C.c_double, C.c_double, C.c_int]
        L.orc_heat_dirichlet.argtypes = [C.POINTER(Grid), C.c_double, C.c_double, C.c_double,
                                         C.c_double, C.c_int, dp, Known, Known, C.c_int]
        L.orc_heat_dirichlet_ws.argtypes = [C.POINTER(Grid), C.c_double, C.c_double, C.c_double,
                                            C.c_double, C.c_int, dp, dp, Known, Known, C.c_int]
        L.orc_first_touch.argtypes = [dp, C.c_size_t, C.c_int]
        L.orc_first_touch.restype = None
        L.orc_pennes_mri.argtypes = [C.POINTER(Grid)] + [C.c_double] * 7 + [dp, dp, C.c_int, dp, C.c_int]
        L.orc_heat_flux.argtypes = [C.POINTER(Grid)] + [C.c_double] * 6 + [C.c_int, C.c_int, dp, Known, Known,
                                                                         Known, C.c_int]
        L.orc_heat_radiation.argtypes = [C.POINTER(Grid)] + [C.c_double] * 7 + [C.c_int, dp, Known, Known,
                                                                              Known, C.c_int]
        L.orc_kheat_tangent.argtypes = [C.POINTER(Grid), dp, dp, C.c_int, dp, dp, C.c_int]
        L.orc_pennes_tissue.argtypes = [C.POINTER(Grid), C.POINTER(Tissue), C.c_int, dp, C.c_int]
        L.orc_pennes_tissue.restype = C.c_int
        L.orc_stencil_width_one.argtypes = [C.POINTER(Grid), C.c_int, dp, C.c_int]
        L.orc_stencil_width_var.argtypes = [C.POINTER(Grid), C.c_int, C.c_int, dp, C.c_int]
        L.orc_kheat_forward.argtypes = [C.POINTER(Grid), dp, C.c_int, dp, dp, C.c_int]
        L.orc_kheat_adjoint.argtypes = [C.POINTER(Grid), dp, C.c_int, dp, dp, dp, dp, dp, C.c_int]
        L.orc_kheat_adjoint_reset.argtypes = L.orc_kheat_adjoint.argtypes
        L.orc_kheat_adjoint_reset.restype = C.c_int
        L.orc_lame.argtypes = [C.POINTER(Grid), C.c_double, C.c_double, C.c_double, C.c_int, dp, dp, C.c_int]
        L.orc_yee.argtypes = [C.POINTER(Grid), C.c_int, dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                              C.c_double, C.c_double, C.c_int]
        for f in ("orc_heat_dirichlet", "orc_heat_dirichlet_ws", "orc_pennes_mri", "orc_stencil_width_one",
                  "orc_stencil_width_var", "orc_kheat_forward", "orc_kheat_adjoint", "orc_lame", "orc_yee"):
            getattr(L, f).restype = C.c_int
        L.orc_time.restype = C.c_double
        L.orc_time.argtypes = [C.POINTER(Grid), C.c_int]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with status {rc}")


def make_grid(n, first=(0.0, 0.0, 0.0), last=(1.0, 1.0, 1.0), tau=0.0, t_start=0.0,
              n_layers=1, dim=3) -> Grid:
    g = Grid()
    nn = (C.c_int * 3)(*n)
    f = (C.c_double * 3)(*first)
    l_ = (C.c_double * 3)(*last)
    lib().orc_grid_init(C.byref(g), dim, nn, f, l_, tau, t_start, n_layers)
    return g


def coords(g: Grid):
    """Coordinates x_p = first_p + h_p * i_p (src/ScaFES_Grid.hpp:721-733),
    broadcastable to (nz, ny, nx)."""
    nx, ny, nz = g.n[0], g.n[1], g.n[2]
    x = g.first[0] + g.h[0] * np.arange(nx, dtype=np.float64)
    y = g.first[1] + g.h[1] * np.arange(ny, dtype=np.float64)
    z = g.first[2] + g.h[2] * np.arange(nz, dtype=np.float64)
    return x[None, None, :], y[None, :, None], z[:, None, None]


def border_mask(g: Grid) -> np.ndarray:
    """Global-border nodes (src/ScaFES_Problem.hpp:3952-3971)."""
    nx, ny, nz = g.n[0], g.n[1], g.n[2]
    L = g.n_layers
    m = np.zeros((nz, ny, nx), dtype=bool)
    m[:L, :, :] = m[-L:, :, :] = True
    m[:, :L, :] = m[:, -L:, :] = True
    m[:, :, :L] = m[:, :, -L:] = True
    return m


def heat_dirichlet(g: Grid, u0, nsteps, coeff_a=1.0, rho_c=1.0, perf_q1=0.0, perf_w=0.0,
                   f_base=None, f_form=0, f_a=1.0, f_b=0.0,
                   g_base=None, g_form=0, g_a=1.0, g_b=0.0, nthreads=0):
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    fk = Known(_p(f_base), f_form, f_a, f_b)
    gk = Known(_p(g_base), g_form, g_a, g_b)
    _check(lib().orc_heat_dirichlet(C.byref(g), coeff_a, rho_c, perf_q1, perf_w, nsteps,
                                    _p(u), fk, gk, nthreads), "heat_dirichlet")
    return u


def first_touched(shape, nthreads=0) -> np.ndarray:
    """An uninitialised float64 array whose pages the OpenMP threads of the
    sweeps have already mapped (zeros)."""
    a = np.empty(shape, dtype=np.float64)
    lib().orc_first_touch(_p(a), a.size, nthreads)
    return a


def heat_dirichlet_ws(g: Grid, u, w, nsteps, coeff_a=1.0, rho_c=1.0, nthreads=0):
    """heat_dirichlet on caller-owned C-contiguous float64 fields u, w (no
    copy, no allocation): returns the array holding iterate nsteps (u for
    even nsteps, w for odd)."""
    for a in (u, w):
        if a.dtype != np.float64 or not a.flags.c_contiguous or a.size != g.n[0] * g.n[1] * g.n[2]:
            raise ValueError("heat_dirichlet_ws needs C-contiguous float64 fields of the grid's size")
    none = Known(None, 0, 1.0, 0.0)
    _check(lib().orc_heat_dirichlet_ws(C.byref(g), coeff_a, rho_c, 0.0, 0.0, nsteps, _p(u), _p(w), none, none,
                                       nthreads), "heat_dirichlet_ws")
    return u if nsteps % 2 == 0 else w


def heat_flux(g: Grid, u0, nsteps, kind, coeff_a=1.0, rho_c=1.0, perf_q1=0.0, perf_w=0.0, lam=1.0,
              alpha=1.0, f=(None, 0, 1.0, 0.0), g_dir=(None, 0, 1.0, 0.0), g_flux=(None, 0, 1.0, 0.0),
              nthreads=0):
    """Flux-condition border (kind 0 Neumann, 1 Cauchy); f, g_dir, g_flux
    are (base, form, a, b) known fields."""
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    keep = [np.ascontiguousarray(k[0], dtype=np.float64) if k[0] is not None else None for k in (f, g_dir, g_flux)]
    ks = [Known(_p(b), k[1], k[2], k[3]) for b, k in zip(keep, (f, g_dir, g_flux))]
    _check(lib().orc_heat_flux(C.byref(g), coeff_a, rho_c, perf_q1, perf_w, lam, alpha, kind, nsteps,
                               _p(u), ks[0], ks[1], ks[2], nthreads), "heat_flux")
    return u


def heat_radiation(g: Grid, u0, nsteps, coeff_a=1.0, rho_c=1.0, perf_q1=0.0, perf_w=0.0, lam=1.0,
                   epsilon=1.0, sigma=1.0, f=(None, 0, 1.0, 0.0), g_dir=(None, 0, 1.0, 0.0),
                   g_flux=(None, 0, 1.0, 0.0), nthreads=0):
    """Radiation border (Radiation.hpp); f, g_dir, g_flux as for heat_flux."""
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    keep = [np.ascontiguousarray(k[0], dtype=np.float64) if k[0] is not None else None for k in (f, g_dir, g_flux)]
    ks = [Known(_p(b), k[1], k[2], k[3]) for b, k in zip(keep, (f, g_dir, g_flux))]
    _check(lib().orc_heat_radiation(C.byref(g), coeff_a, rho_c, perf_q1, perf_w, lam, epsilon, sigma, nsteps,
                                    _p(u), ks[0], ks[1], ks[2], nthreads), "heat_radiation")
    return u


def pennes_mri(g: Grid, u0, nsteps, rho, c, k, rho_b, c_b, omega, t_blood, q, g_bdry, nthreads=0):
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    q = np.ascontiguousarray(q, dtype=np.float64)
    gb = np.ascontiguousarray(g_bdry, dtype=np.float64)
    _check(lib().orc_pennes_mri(C.byref(g), rho, c, k, rho_b, c_b, omega, t_blood, _p(q), _p(gb),
                                nsteps, _p(u), nthreads), "pennes_mri")
    return u


TISSUE_FIELDS = ("rho", "c", "k", "rho_b", "c_b", "omega", "t_blood", "q")


def pennes_tissue(g: Grid, u0, nsteps, fields: dict, surface=None, zmax_kind=0, q_bc=0.0, q_skull=0.0,
                  h_conv=0.0, t_amb=0.0, epsilon=0.0, sigma=5.670373e-8, g_bdry=None, nthreads=0):
    """The reference's tissue examples (orc_pennes_tissue): ``fields`` maps
    each name of TISSUE_FIELDS to an array over the nodes (or a scalar);
    g_bdry given => Dirichlet border from it, else the examples' flux
    border."""
    shape = (g.n[2], g.n[1], g.n[0])
    keep = {}
    for name in TISSUE_FIELDS:
        keep[name] = np.ascontiguousarray(np.broadcast_to(np.asarray(fields.get(name, 0.0), dtype=np.float64),
                                                          shape))
    if surface is not None:
        keep["surface"] = np.ascontiguousarray(np.broadcast_to(np.asarray(surface, dtype=np.float64), shape))
    if g_bdry is not None:
        keep["g_bdry"] = np.ascontiguousarray(np.broadcast_to(np.asarray(g_bdry, dtype=np.float64), shape))
    ts = Tissue(*[_p(keep[n]) for n in TISSUE_FIELDS], _p(keep.get("surface")), zmax_kind, q_bc, q_skull,
                h_conv, t_amb, epsilon, sigma, 1 if g_bdry is not None else 0, _p(keep.get("g_bdry")))
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    _check(lib().orc_pennes_tissue(C.byref(g), C.byref(ts), nsteps, _p(u), nthreads), "pennes_tissue")
    return u


def tumour_fields(g: Grid, P: dict) -> dict:
    """Per-node fields of the tumour example (TumorHeatEqnFDM.hpp:234-252):
    omega and Q from the sphere test, the tissue constants everywhere;
    P holds the example's Parameters (RHO, C, K, ... as in its .ini)."""
    x, y, z = coords(g)
    radius = P["DIAMETER"] / 2.0
    centre = (g.last[0] / 2.0, g.last[1] / 2.0, g.last[2] - P["DEPTH"])
    d = 0.0 + (x - centre[0]) * (x - centre[0])
    d = d + (y - centre[1]) * (y - centre[1])
    d = d + (z - centre[2]) * (z - centre[2])
    inside = np.broadcast_to(d <= radius * radius, (g.n[2], g.n[1], g.n[0]))
    return {"rho": P["RHO"], "c": P["C"], "k": P["K"], "rho_b": P["RHO_B"], "c_b": P["C_PB"],
            "omega": np.where(inside, P["OMEGA_B_TUMOR"], P["OMEGA_B_BRAIN"]),
            "t_blood": P["T_A"], "q": np.where(inside, P["Q_TUMOR"], P["Q_BRAIN"])}


def stencil_width_one(g: Grid, u0, nsteps, nthreads=0):
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    _check(lib().orc_stencil_width_one(C.byref(g), nsteps, _p(u), nthreads), "stencil_width_one")
    return u


def stencil_width_var(g: Grid, u0, bw, nsteps, nthreads=0):
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    _check(lib().orc_stencil_width_var(C.byref(g), bw, nsteps, _p(u), nthreads), "stencil_width_var")
    return u


def kheat_forward(g: Grid, k, u0, nsteps, keep_traj=False, nthreads=0):
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    k = np.ascontiguousarray(k, dtype=np.float64)
    traj = np.empty((nsteps + 1,) + u.shape, dtype=np.float64) if keep_traj else None
    _check(lib().orc_kheat_forward(C.byref(g), _p(k), nsteps, _p(u), _p(traj), nthreads), "kheat_forward")
    return (u, traj) if keep_traj else u


def kheat_tangent(g: Grid, k, dk, u0, du0, nsteps, nthreads=0):
    """Forward-mode AD of the variable-k solve: (u_T, du_T) along (dk, du0)."""
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    du = np.ascontiguousarray(du0, dtype=np.float64).copy()
    k = np.ascontiguousarray(k, dtype=np.float64)
    dk = np.ascontiguousarray(dk, dtype=np.float64)
    _check(lib().orc_kheat_tangent(C.byref(g), _p(k), _p(dk), nsteps, _p(u), _p(du), nthreads), "kheat_tangent")
    return u, du


def kheat_adjoint(g: Grid, k, traj, target, nthreads=0, reset_border=False):
    """J, dJ/dk, dJ/du0 of J = 0.5 ||u_T - target||^2 for the flux-form
    solve with trajectory traj.  reset_border: the border is reset to fixed
    values every step (a Dirichlet border) instead of held at u0's values;
    u0's border then enters the first step only."""
    nsteps = traj.shape[0] - 1
    k = np.ascontiguousarray(k, dtype=np.float64)
    target = np.ascontiguousarray(target, dtype=np.float64)
    gk = np.empty_like(k)
    gu = np.empty_like(k)
    j = C.c_double(0.0)
    fn = lib().orc_kheat_adjoint_reset if reset_border else lib().orc_kheat_adjoint
    _check(fn(C.byref(g), _p(k), nsteps, _p(traj), _p(target), _p(gk), _p(gu), C.byref(j), nthreads),
           "kheat_adjoint")
    return j.value, gk, gu


def lame(g: Grid, u, uprev, nsteps, lam, mu, rho, nthreads=0):
    """u, uprev: arrays (3, nz, ny, nx); returns (u^nsteps, u^(nsteps-1))."""
    u = np.ascontiguousarray(u, dtype=np.float64).copy()
    up = np.ascontiguousarray(uprev, dtype=np.float64).copy()
    _check(lib().orc_lame(C.byref(g), lam, mu, rho, nsteps, _p(u), _p(up), nthreads), "lame")
    return u, up


def yee(g: Grid, fields, nsteps, src, amp, t0, w, freq, nthreads=0):
    """fields: array (6, nz, ny, nx) = Ex, Ey, Ez, Hx, Hy, Hz."""
    f = np.ascontiguousarray(fields, dtype=np.float64).copy()
    _check(lib().orc_yee(C.byref(g), nsteps, _p(f), int(src[0]), int(src[1]), int(src[2]), amp, t0, w, freq,
                         nthreads), "yee")
    return f


# ---- reference-driver programs (oracle/_ref) ---------------------------------

def ref_available(name: str) -> bool:
    return (REF_DIR / name).exists() and os.access(REF_DIR / name, os.X_OK)


def run_ref(name: str, n, nsteps, workdir, t_start=0.0, t_end=1.0, tau=0.0,
            first=(0.0, 0.0, 0.0), last=(1.0, 1.0, 1.0), inputs=None, extra=(), nfields=1,
            threads=1, n_layers=1) -> np.ndarray:
    """Runs oracle/_ref/<name> and returns its final field(s), shape
    (nfields, nz, ny, nx) (or (nz, ny, nx) for one field)."""
    workdir = Path(workdir)
    out = workdir / f"{name}.out.bin"
    args = [str(REF_DIR / name), *map(str, n), str(nsteps), repr(float(t_start)), repr(float(t_end)),
            repr(float(tau)), *map(lambda v: repr(float(v)), first), *map(lambda v: repr(float(v)), last),
            str(out)]
    if inputs is not None:
        inp = workdir / f"{name}.in.bin"
        np.ascontiguousarray(inputs, dtype=np.float64).tofile(inp)
        args.append(str(inp))
    args += [repr(float(v)) for v in extra]
    env = dict(os.environ, OMP_NUM_THREADS=str(threads), HARNESS_NLAYERS=str(n_layers))
    subprocess.run(args, check=True, capture_output=True, env=env)
    nz, ny, nx = n[2], n[1], n[0]
    v = np.fromfile(out, dtype=np.float64)
    v = v.reshape((nfields, nz, ny, nx))
    return v[0] if nfields == 1 else v
