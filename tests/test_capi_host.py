"""Host-side checks of the C ABI that need no GPU: the library loads, it
exports every function include/*.h declares, and invalid configurations are
rejected with a status code (argument checking happens before any CUDA call).
"""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(scafes_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_functions():
    names = declared_functions()
    for expected in ("scafes_gpu_create", "scafes_gpu_upload", "scafes_gpu_step",
                     "scafes_gpu_download", "scafes_gpu_destroy", "scafes_gpu_last_error"):
        assert expected in names


def test_library_exports_every_declared_symbol(native):
    L = native.lib()
    missing = [n for n in declared_functions() if not hasattr(L, n)]
    assert not missing, f"declared but not exported: {missing}"


def _create(M, **kw):
    cfg = M.make_cfg((8, 8, 8), tau=1e-3, precision="f64", c0=0.4, cp=(0.1, 0.1, 0.1))
    for k, v in kw.items():
        if k == "n_nodes":
            cfg.n_nodes[:] = v
        else:
            setattr(cfg, k, v)
    h = C.c_void_p()
    rc = M.lib().scafes_gpu_create(C.byref(cfg), C.byref(h))
    return rc, h


@pytest.mark.parametrize("kw,code", [
    (dict(dim=2), -4),
    (dict(n_nodes=(2, 8, 8)), -1),
    (dict(n_nodes=(8, 8, 0)), -1),
    (dict(n_layers_at_border=0), -1),
    (dict(n_layers_at_border=5), -1),             # more than half of the smallest axis (8)
    (dict(n_layers_at_border=2, border=1), -4),   # the mirror rule has one layer
    (dict(precision=17), -4),
    (dict(border=9), -4),
    (dict(tile=5), -1),
    (dict(tile=-1), -1),
])
def test_invalid_config_rejected(native, kw, code):
    rc, h = _create(native, **kw)
    assert rc == code
    assert not h.value
    assert native.lib().scafes_last_error()  # a message is recorded


def test_null_arguments(native):
    L = native.lib()
    h = C.c_void_p()
    assert L.scafes_gpu_create(None, C.byref(h)) == -1
    assert L.scafes_gpu_step(None, 1) == -1
    assert L.scafes_gpu_upload(None, 0, None, 0) == -1
    assert L.scafes_gpu_download(None, 0, None, 0) == -1
    L.scafes_gpu_destroy(None)  # no-op


def test_backward_entries_check_arguments_first(native):
    """The backward entry, its kept initial iterate and the adjoint handle's
    hooks refuse a NULL handle with SCAFES_ERR_ARG before any CUDA call."""
    L = native.lib()  # the binding declares the plain handle's entries
    L.scafes_adj_set_conductivity_uniform.argtypes = [C.c_void_p, C.c_double]
    L.scafes_adj_inject_status.argtypes = [C.c_void_p, C.c_int]
    assert L.scafes_gpu_adjoint(None, None, None, None, 8) == -1
    assert L.scafes_gpu_keep_initial(None, 1) == -1
    assert L.scafes_adj_set_conductivity_uniform(None, 1.0) == -1
    assert L.scafes_adj_inject_status(None, -6) == -1
    assert L.scafes_last_error()


def test_heat_coeffs_helper(native):
    M = native
    n, tau = (11, 21, 31), 1e-5
    cfg = M.make_cfg(n, last=(1.0, 2.0, 3.0), tau=tau, heat=(0.7, 2.0, 0.25))
    h = [(l - 0.0) / (m - 1) for l, m in zip((1.0, 2.0, 3.0), n)]
    cp = [tau * 0.7 / (hh * hh) for hh in h]
    assert list(cfg.cp) == pytest.approx(cp, rel=1e-15)
    assert cfg.c0 == pytest.approx(1.0 - 2.0 * sum(cp) - tau * 0.25, rel=1e-15)
    assert cfg.cf == pytest.approx(tau / 2.0, rel=1e-15)


def test_border_forms_flux_match_reference_rules(native):
    """scafes_border_forms_flux on the host: Dirichlet at min faces, the
    mirrored neighbour and the flux weight at max faces (Neumann.hpp /
    Cauchy.hpp / Radiation.hpp of the system tests)."""
    M = native
    n = (10, 8, 6)
    cfg = M.make_cfg(n, tau=1e-3, border=M.BORDER_TABLE, heat=(1.0, 1.0, 0.0))
    h = [1.0 / (m - 1) for m in n]
    for kind, alpha in ((M.FLUX_NEUMANN, 0.0), (M.FLUX_CAUCHY, 0.7), (M.FLUX_RADIATION, 0.3)):
        F = M.border_forms_flux(cfg, kind, 2.0, alpha)
        for m in range(1, 64):
            r = F[m]
            if m & (1 | 4 | 16):
                assert (r.cu, list(r.cn), r.cf, r.cg_old, r.cg_new, r.cu4) == (0.0, [0.0] * 6, 0.0, 0.0, 1.0, 0.0)
                continue
            flux = 0.0
            for p in range(3):
                if (m >> (2 * p + 1)) & 1:
                    assert r.cn[2 * p] == 2.0 * cfg.cp[p] and r.cn[2 * p + 1] == 0.0
                    flux += cfg.cp[p] * (2.0 * h[p] / 2.0)
                else:
                    assert r.cn[2 * p] == r.cn[2 * p + 1] == cfg.cp[p]
            assert r.cf == cfg.cf and r.cg_new == 0.0
            if kind == M.FLUX_NEUMANN:
                assert abs(r.cg_old + flux) < 1e-15 and r.cu == cfg.c0 and r.cu4 == 0.0
            elif kind == M.FLUX_CAUCHY:
                assert abs(r.cg_old - flux) < 1e-15 and abs(r.cu - (cfg.c0 - alpha * flux)) < 1e-15
                assert r.cu4 == 0.0
            else:
                assert abs(r.cg_old - flux) < 1e-15 and r.cu == cfg.c0
                assert abs(r.cu4 + alpha * flux) < 1e-15
    with pytest.raises(M.ScafesError):
        M.border_forms_flux(cfg, 7, 1.0, 1.0)
