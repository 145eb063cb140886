"""Failure detection on the GPU without a fault (the pool forbids faulting,
trapping or hanging a GPU): the bounded device wait that guards every TMA
load of the sweep kernels gives up on an mbarrier that never completes and
reports SCAFES_ERR_TIMEOUT in the status word, after its limit and not much
later; a status set on a handle (as a sweep that gave up sets it) makes the
later sweeps skip their work and the next download report it once; the
context stays usable and later runs match the oracle."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import cases
import oracle as O

pytestmark = pytest.mark.gpu

TIMEOUT = -6


def heat_problem(n, seed=3):
    rng = np.random.default_rng(seed)
    shape = (n[2], n[1], n[0])
    tau = 0.9 / (2.0 * sum((m - 1) ** 2 for m in n))
    return rng.uniform(-1.0, 1.0, shape), tau


def run_and_check(M, n, T):
    u0, tau = heat_problem(n)
    with M.Plain(M.make_cfg(n, tau=tau, heat=(1.0, 1.0, 0.0))) as p:
        p.upload(M.FIELD_U, u0)
        p.step(T)
        u = p.download()
    assert cases.rel_err(u, O.heat_dirichlet(O.make_grid(n, tau=tau), u0, T)) <= 1e-12


@pytest.mark.parametrize("limit_us", [20000, 200000])
def test_bounded_wait_gives_up_and_reports(gpu, limit_us):
    M = gpu
    fn = M.lib().scafes_probe_wait_timeout
    fn.argtypes = [C.c_uint, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    fn.restype = C.c_int
    st, ms = C.c_int(), C.c_double()
    assert fn(limit_us, C.byref(st), C.byref(ms)) == 0
    assert st.value == TIMEOUT
    # gave up after the limit, and within one suspension hint plus slack
    assert limit_us / 1000.0 <= ms.value <= limit_us / 1000.0 + 50.0
    run_and_check(M, (24, 20, 18), 10)  # the context is still usable


def test_status_skips_sweeps_and_is_reported_once(gpu):
    M = gpu
    n, T = (24, 20, 18), 6
    u0, tau = heat_problem(n)
    inj = M.lib().scafes_gpu_inject_status
    inj.argtypes = [C.c_void_p, C.c_int]
    with M.Plain(M.make_cfg(n, tau=tau, heat=(1.0, 1.0, 0.0))) as p:
        p.upload(M.FIELD_U, u0)
        assert inj(p.h, TIMEOUT) == 0
        p.step(T)                                 # the sweeps see the status and return at once
        with pytest.raises(M.ScafesError) as ex:
            p.download()
        assert ex.value.code == TIMEOUT
        p.upload(M.FIELD_U, u0)                   # the status was cleared: a fresh run is correct
        p.step(T)
        u = p.download()
    assert cases.rel_err(u, O.heat_dirichlet(O.make_grid(n, tau=tau), u0, T)) <= 1e-12


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
def test_adjoint_status_is_reported_and_cleared(gpu, prec):
    """An adjoint handle's status word: set (as a pair step that gave up
    sets it), the next forward solve and the next gradient each report it
    once -- the pair steps skip their work meanwhile -- and the runs after
    that give the same bits as on a fresh handle."""
    M = gpu
    n, T = (40, 18, 36), 8
    rng = np.random.default_rng(9)
    shape = (n[2], n[1], n[0])
    k = np.exp(0.3 * rng.standard_normal(shape))
    u0, target = rng.uniform(-1.0, 1.0, shape), rng.uniform(-1.0, 1.0, shape)
    tau = 0.4 / (2.0 * float(k.max()) * sum((m - 1) ** 2 for m in n))
    inj = M.lib().scafes_adj_inject_status
    inj.argtypes = [C.c_void_p, C.c_int]
    with M.Adjoint(n, tau, 4, precision=prec) as a:
        a.set_conductivity(k)
        uT_ref = a.forward(u0, T)
        J_ref, gk_ref, gu_ref = a.gradient(u0, target, T)
    with M.Adjoint(n, tau, 4, precision=prec) as a:
        a.set_conductivity(k)
        assert inj(a.h, TIMEOUT) == 0
        with pytest.raises(M.ScafesError) as ex:
            a.forward(u0, T)
        assert ex.value.code == TIMEOUT
        assert np.array_equal(a.forward(u0, T), uT_ref)
        assert inj(a.h, TIMEOUT) == 0
        with pytest.raises(M.ScafesError) as ex:
            a.gradient(u0, target, T)
        assert ex.value.code == TIMEOUT
        J, gk, gu = a.gradient(u0, target, T)
    assert J == J_ref and np.array_equal(gk, gk_ref) and np.array_equal(gu, gu_ref)
