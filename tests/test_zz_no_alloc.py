"""The allocation-free max-norm check (scafes_err_linf_noalloc).

This entry point exists for callers that must not allocate device memory
where they check the error -- a time loop being recorded into a CUDA graph,
a serving loop that forbids cudaMalloc after start-up, a host whose device
memory all comes from its own pool.  It keeps its partial maxima in a fixed
array inside the library instead of a buffer made by scafes_gpu_create.

The test checks it through the C ABI against the handle-based
scafes_gpu_err_linf on the same data, for two calls in a row (the second
call must not see the first call's partial maxima), and that sizes beyond
the fixed scratch are refused.  It lives in its own file, collected last, and
passes both alone in a fresh process and after the other tests.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(M):
    fn = M.lib().scafes_err_linf_noalloc
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return fn


def _handle_err(M, u, e):
    n = (u.shape[2], u.shape[1], u.shape[0])
    cfg = M.make_cfg(n, tau=1e-3, precision="f64", heat=(1.0, 1.0, 0.0))
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_E_A, e)
        p.upload(M.FIELD_U, u)
        return p.err_linf()


def test_noalloc_matches_handle_two_calls(gpu):
    torch = pytest.importorskip("torch")
    M = gpu
    fn = _noalloc(M)
    rng = np.random.default_rng(42)
    # The second call covers fewer CTAs than the first and has smaller values:
    # reading any partial maximum left by the first call would show.
    cases = [(40, 64, 128), (29, 33, 70)]
    for k, shape in enumerate(cases):
        u = rng.uniform(-1.0, 1.0, shape)
        e = u + rng.uniform(-1e-9, 1e-9, shape) * (10.0 ** -k)
        if k == 1:
            u *= 0.25
            e *= 0.25
        du = torch.from_numpy(u).cuda()
        de = torch.from_numpy(e).cuda()
        out = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = fn(du.data_ptr(), de.data_ptr(), u.size, out.data_ptr(), None)
        assert rc == 0, M.lib().scafes_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        ref_err, ref_max = _handle_err(M, u, e)
        assert got[0] == pytest.approx(ref_err, rel=1e-12, abs=0.0)
        assert got[1] == pytest.approx(ref_max, rel=1e-12, abs=0.0)
        assert got[0] == pytest.approx(float(np.max(np.abs(u - e))), rel=1e-12)


def test_noalloc_rejects_oversize_and_null(gpu):
    torch = pytest.importorskip("torch")
    M = gpu
    fn = _noalloc(M)
    buf = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = buf.data_ptr()
    too_big = 16384 * 32768 + 1
    assert fn(p, p, too_big, p, None) == -1
    assert b"scratch" in M.lib().scafes_last_error()
    assert fn(None, p, 4, p, None) == -1
    assert fn(p, p, 0, p, None) == -1
