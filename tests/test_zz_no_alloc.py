"""The allocation-free max-norm check (scafes_err_linf_noalloc).

This entry point exists for callers that must not allocate device memory
where they check the error -- a serving loop that forbids cudaMalloc after
start-up, a host whose device memory all comes from its own pool.  It keeps its partial maxima in a fixed
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


_RESET_CHILD = r"""
import ctypes as C
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import masterthesis_gb300 as M

# The library first, then the CUDA runtime it links (same soname, so the
# same runtime instance).
L = M.lib()
rt = None
for name in ("libcudart.so.13", "libcudart.so", "libcudart.so.12"):
    try:
        rt = C.CDLL(name)
        break
    except OSError:
        continue
assert rt is not None, "libcudart not found"
rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
rt.cudaFree.argtypes = [C.c_void_p]
fn = M.lib().scafes_err_linf_noalloc
fn.argtypes = [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_void_p]
fn.restype = C.c_int
rng = np.random.default_rng(7)


def one_call(n, scale):
    u = rng.uniform(-scale, scale, n)
    e = u + rng.uniform(-1e-9, 1e-9, n)
    bufs = [C.c_void_p() for _ in range(3)]
    for b, size in zip(bufs, (8 * n, 8 * n, 16)):
        assert rt.cudaMalloc(C.byref(b), size) == 0
    assert rt.cudaMemcpy(bufs[0], u.ctypes.data, 8 * n, 1) == 0
    assert rt.cudaMemcpy(bufs[1], e.ctypes.data, 8 * n, 1) == 0
    rc = fn(bufs[0], bufs[1], n, bufs[2], None)
    assert rc == 0, M.lib().scafes_last_error()
    assert rt.cudaDeviceSynchronize() == 0
    out = np.empty(2)
    assert rt.cudaMemcpy(out.ctypes.data, bufs[2], 16, 2) == 0
    for b in bufs:
        rt.cudaFree(b)
    assert out[0] == np.max(np.abs(u - e)) and out[1] == np.max(np.abs(e)), (out, n)


one_call(300_000, 1.0)
# A new primary context: the module (and its scratch array) is loaded again.
assert rt.cudaDeviceReset() == 0
one_call(200_000, 0.5)
one_call(100_000, 0.25)
print("RESET_OK")
"""


def test_noalloc_after_context_reset(gpu):
    """After cudaDeviceReset the library's module is loaded again in a new
    context; the entry point must look its scratch address up again instead
    of reusing the old context's.  Runs in a child process (plain CUDA
    runtime calls, no torch) so that this process keeps its context."""
    import subprocess
    import sys
    from pathlib import Path

    root = str(Path(__file__).resolve().parents[1])
    res = subprocess.run([sys.executable, "-c", _RESET_CHILD, root], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0 and "RESET_OK" in res.stdout, res.stdout + res.stderr
