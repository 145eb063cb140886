"""The FP64 sweep adds its neighbour sums on the integer pipe
(masterthesis_gb300/csrc/dadd_int.cuh): every such sum must carry the FP64
adder's exact bits (round to nearest even), and the sweep must equal, bit for
bit, a C model of its operation order built on the host's FP64 adder and
fma().

CPU: the adder compiled for the host against its FP64 adder on seeded inputs
(ties, carries into the exponent, the overflow threshold, subnormal and
opposite-sign operands it must hand back); the device entry's argument
checks.  GPU: the same adder on the device against numpy's FP64 addition,
and whole sweeps against the C model on fields that keep it on the integer
path and fields that send warps to the FP64 fallback.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
NATIVE = ROOT / "tests" / "native"


def _build(tmp_path_factory, src: str, out: str, extra=()) -> Path:
    d = tmp_path_factory.mktemp("native")
    exe = d / out
    subprocess.run(["gcc" if src.endswith(".c") else "g++", "-O2", "-ffp-contract=off", *extra,
                    "-o", str(exe), str(NATIVE / src), "-lm"], check=True)
    return exe


@pytest.fixture(scope="module")
def adder_check(tmp_path_factory):
    return _build(tmp_path_factory, "dadd_int_check.cpp", "dadd_int_check")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_integer_adder_matches_fp64_adder_on_host(adder_check, seed):
    res = subprocess.run([str(adder_check), "4000000", str(seed)], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout
    n, fast, bad = (int(v) for v in res.stdout.split()[-3:])
    assert bad == 0 and n == 4000000
    assert fast > n // 3  # most generated pairs lie on the integer path


def test_probe_entry_checks_arguments(native):
    L = native.lib()
    a = (C.c_ulonglong * 4)()
    ok = (C.c_ubyte * 4)()
    assert L.scafes_probe_dadd_int(a, a, a, ok, 0) == -1
    assert L.scafes_probe_dadd_int(None, a, a, ok, 4) == -1
    assert L.scafes_probe_dadd_int(a, a, a, ok, (1 << 26) + 1) == -1


# ---- device ------------------------------------------------------------------

def _bits(sign, exp, frac):
    return (np.asarray(sign, np.uint64) << np.uint64(63)) | (np.asarray(exp, np.uint64) << np.uint64(52)) | (
        np.asarray(frac, np.uint64) & np.uint64(0x000FFFFFFFFFFFFF))


def _shaped(rng, n):
    """Significands whose low bits are all zeros or all ones."""
    f = rng.integers(0, 2 ** 63, n, dtype=np.uint64)
    k = rng.integers(0, 53, n).astype(np.uint64)
    mask = (np.uint64(1) << k) - np.uint64(1)
    kind = rng.integers(0, 4, n)
    return np.where(kind == 0, f & ~mask, np.where(kind == 1, f | mask, np.where(kind == 2, mask, f)))


def adder_cases(seed, n):
    rng = np.random.default_rng(seed)
    s = rng.integers(0, 2, n).astype(np.uint64)
    ea = rng.integers(1, 2047, n).astype(np.int64)
    d = np.where(rng.integers(0, 4, n) > 0, rng.integers(0, 12, n), rng.integers(0, 72, n))
    eb = np.maximum(ea - d, 1)
    a1, b1 = _bits(s, ea, rng.integers(0, 2 ** 63, n, dtype=np.uint64)), _bits(s, eb, _shaped(rng, n))
    ea2 = np.where(rng.integers(0, 2, n) == 1, rng.integers(2040, 2048, n), rng.integers(0, 8, n))
    eb2 = np.maximum(ea2 - rng.integers(0, 9, n), 0)
    s2 = s ^ (rng.integers(0, 8, n) == 0).astype(np.uint64)
    a2, b2 = _bits(s, ea2, _shaped(rng, n)), _bits(s2, eb2, _shaped(rng, n))
    a3 = rng.integers(0, 2 ** 64 - 1, n, dtype=np.uint64, endpoint=True)
    b3 = rng.integers(0, 2 ** 64 - 1, n, dtype=np.uint64, endpoint=True)
    a = np.concatenate([a1, a2, a3])
    b = np.concatenate([b1, b2, b3])
    swap = rng.integers(0, 2, a.size) == 1
    return np.where(swap, b, a), np.where(swap, a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("seed", [11, 12])
def test_integer_adder_matches_fp64_adder_on_device(gpu, seed):
    M = gpu
    a, b = adder_cases(seed, 1 << 21)
    out = np.empty_like(a)
    ok = np.empty(a.size, np.uint8)
    ptr = lambda x, t: x.ctypes.data_as(C.POINTER(t))  # noqa: E731
    rc = M.lib().scafes_probe_dadd_int(ptr(a, C.c_ulonglong), ptr(b, C.c_ulonglong), ptr(out, C.c_ulonglong),
                                       ptr(ok, C.c_ubyte), a.size)
    assert rc == 0
    ea = (a >> np.uint64(52)) & np.uint64(0x7FF)
    eb = (b >> np.uint64(52)) & np.uint64(0x7FF)
    big, small = np.maximum(ea, eb), np.minimum(ea, eb)
    same = (a >> np.uint64(63)) == (b >> np.uint64(63))
    expect_ok = same & (small >= 1) & (small <= 2035) & (big - small <= 10)
    assert np.array_equal(ok.astype(bool), expect_ok)
    with np.errstate(over="ignore", invalid="ignore"):
        want = (a.view(np.float64) + b.view(np.float64)).view(np.uint64)
    sel = ok.astype(bool)
    assert sel.sum() > a.size // 5
    bad = np.flatnonzero(out[sel] != want[sel])
    assert bad.size == 0, [(hex(int(a[sel][i])), hex(int(b[sel][i]))) for i in bad[:4]]


@pytest.fixture(scope="module")
def star_model(tmp_path_factory):
    so = _build(tmp_path_factory, "star7_order.c", "star7_order.so", extra=("-shared", "-fPIC"))
    lib = C.CDLL(str(so))
    dp = C.POINTER(C.c_double)
    lib.star7_sweep_f64.argtypes = [dp, dp, C.c_int, C.c_int, C.c_int] + [C.c_double] * 5
    lib.star7_vc_sweep_f64.argtypes = [dp, dp, dp, dp, C.c_int, C.c_int, C.c_int] + [C.c_double] * 4
    return lib


def _model_step(lib, u, coeffs, border=0.0):
    nz, ny, nx = u.shape
    u = np.ascontiguousarray(u)
    out = np.empty_like(u)
    dp = C.POINTER(C.c_double)
    lib.star7_sweep_f64(u.ctypes.data_as(dp), out.ctypes.data_as(dp), nx, ny, nz, *coeffs, border)
    return out


def _model_vc_step(lib, u, c0f, caf, cp, border=0.0):
    nz, ny, nx = u.shape
    u = np.ascontiguousarray(u)
    out = np.empty_like(u)
    dp = C.POINTER(C.c_double)
    lib.star7_vc_sweep_f64(u.ctypes.data_as(dp), c0f.ctypes.data_as(dp), caf.ctypes.data_as(dp),
                           out.ctypes.data_as(dp), nx, ny, nz, *cp, border)
    return out


KINDS = ["smooth", "signed", "ties", "wide"]


def _fields(kind, shape, rng):
    nz, ny, nx = shape
    if kind == "smooth":  # one sign, slowly varying: the integer path throughout
        z, y, x = np.meshgrid(*(np.linspace(0.05, 0.95, m) for m in shape), indexing="ij")
        return np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z) + 1e-3 * rng.random(shape)
    if kind == "signed":  # opposite-sign neighbours: warps fall back to FP64 adds
        return rng.uniform(-1.0, 1.0, shape)
    if kind == "ties":  # 53-bit integers: every odd neighbour sum is a rounding tie
        return rng.integers(2 ** 52, 2 ** 53, shape).astype(np.float64)
    if kind == "wide":  # exponents over the whole range, some zeros and subnormals
        v = np.exp2(rng.uniform(-1070.0, 1020.0, shape)) * rng.uniform(1.0, 2.0, shape)
        v[rng.random(shape) < 0.01] = 0.0
        sub = rng.random(shape) < 0.01
        v[sub] = 5e-324 * rng.integers(1, 2 ** 40, int(sub.sum()))
        return v
    raise ValueError(kind)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("tile", [0, 1, 2, 3, 4])
def test_f64_sweep_bitwise_equals_operation_order_model(gpu, star_model, kind, tile):
    M = gpu
    n = (70, 37, 29)
    shape = (n[2], n[1], n[0])
    rng = np.random.default_rng(10 * KINDS.index(kind) + tile)
    coeffs = (0.31, 0.11, 0.09, 0.145)  # c0, cx, cy, cz: distinct per axis
    u = _fields(kind, shape, rng)
    cfg = M.make_cfg(n, tau=1e-3, precision="f64", c0=coeffs[0], cp=coeffs[1:], tile=tile)
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_U, u)
        p.set_temporal_depth(1)
        for _ in range(3):
            p.step(1)
            got = p.download()
            want = _model_step(star_model, u, coeffs)
            assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), kind
            u = got


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["smooth", "signed"])
def test_f64_depth2_sweep_bitwise_equals_operation_order_model(gpu, star_model, kind):
    M = gpu
    n = (64, 48, 40)
    shape = (n[2], n[1], n[0])
    rng = np.random.default_rng(5)
    coeffs = (0.31, 0.11, 0.09, 0.145)
    u = _fields(kind, shape, rng)
    cfg = M.make_cfg(n, tau=1e-3, precision="f64", c0=coeffs[0], cp=coeffs[1:])
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_U, u)
        p.set_temporal_depth(2)
        p.step(4)
        got = p.download()
    for _ in range(4):
        u = _model_step(star_model, u, coeffs)
    assert np.array_equal(got.view(np.uint64), u.view(np.uint64)), kind


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["smooth", "signed", "wide"])
@pytest.mark.parametrize("tile", [1, 2, 3, 4])
def test_f64_variable_coefficient_sweep_bitwise_equals_model(gpu, star_model, kind, tile):
    """The variable-coefficient sweep (per-node C0 and CA) adds its sums on
    the integer pipe too: bit for bit against the C model of its order."""
    M = gpu
    n = (45, 33, 21)
    shape = (n[2], n[1], n[0])
    rng = np.random.default_rng(100 + 10 * KINDS.index(kind) + tile)
    cp = (0.11, 0.09, 0.145)
    u = _fields(kind, shape, rng)
    c0f = rng.uniform(0.3, 0.5, shape)
    caf = rng.uniform(0.6, 1.2, shape)
    cfg = M.make_cfg(n, tau=1e-3, precision="f64", c0=1.0, cp=cp, cf=1.0, tile=tile)
    with M.Plain(cfg) as p:
        p.upload(M.FIELD_C0, c0f)
        p.upload(M.FIELD_CA, caf)
        p.upload(M.FIELD_U, u)
        for _ in range(3):
            p.step(1)
            got = p.download()
            want = _model_vc_step(star_model, u, c0f, caf, cp)
            assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), kind
            u = got


@pytest.mark.gpu
def test_f64_sweep_bitwise_at_full_size(gpu, star_model):
    """The benchmark's 512^3 field (sine mode plus noise, Dirichlet 0), two
    sweeps with the default tile, each bit for bit against the C model."""
    from masterthesis_gb300.workloads import heat_sine_noise, heat_tau
    M = gpu
    n = (512, 512, 512)
    tau = heat_tau(n)
    cp = tuple(tau * (m - 1) ** 2 for m in n)  # tau / h^2 per axis on the unit cube
    c0 = 1.0 - 2.0 * sum(cp)
    u = heat_sine_noise(n)
    with M.Plain(M.make_cfg(n, tau=tau, precision="f64", c0=c0, cp=cp)) as p:
        p.upload(M.FIELD_U, u)
        for _ in range(2):
            p.step(1)
            got = p.download()
            want = _model_step(star_model, u, (c0,) + cp)
            assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
            u = got
