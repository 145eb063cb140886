"""Linear multi-field stencils with a leapfrog phase (scafes_lin_*): the
device form of callbacks that couple several unknown fields.  Checked with
the plain Yee cavity (six fields, H half step then E step) against the
oracle's orc_yee without a source: the rules applied on the CPU, the rules
the drop-in records from a ScaFES class, and the CUDA kernel through the C
ABI and through the drop-in.  Tolerance: 1e-12 relative max-norm (FP64;
the kernel sums the terms in another order than the oracle)."""
from __future__ import annotations

import ctypes as C
import subprocess

import numpy as np
import pytest

import cases
import oracle as O
from dropin.build import HERE, compile_cpp, read_device_form


def yee_case(n, seed=3):
    h = 1.0 / (n[0] - 1)
    last = tuple((m - 1) * h for m in n)
    tau = 0.5 * h / np.sqrt(3.0)
    f0 = np.random.default_rng(seed).uniform(-1.0, 1.0, (6, n[2], n[1], n[0]))
    return last, tau, tau / h, f0


def apply_rules(rules, f, n_phases, T):
    """The rules applied on the CPU (numpy, test helper)."""
    nz, ny, nx = f.shape[1:]
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cls = ((x == 0) * 1 | (x == nx - 1) * 2 | (y == 0) * 4 | (y == ny - 1) * 8 | (z == 0) * 16 |
           (z == nz - 1) * 32)
    classes = np.unique(cls)
    f = f.copy()
    for _ in range(T):
        for ph in range(1, n_phases + 1):
            out = np.empty_like(f)
            for fld in range(f.shape[0]):
                for c in classes:
                    m = cls == c
                    v = np.zeros(int(m.sum()))
                    for s, dx, dy, dz, w in rules[(ph, fld, int(c))]:
                        v = v + w * f[s][z[m] + dz, y[m] + dy, x[m] + dx]
                    out[fld][m] = v
            f = out
    return f


def test_yee_rules_on_cpu_match_oracle():
    n, T = (9, 8, 7), 12
    last, tau, ch, f0 = yee_case(n)
    got = apply_rules(cases.yee_lin_rules(ch), f0, 2, T)
    ref = O.yee(O.make_grid(n, last=last, tau=tau), f0, T, (0, 0, 0), 0.0, 1.0, 1.0, 1.0)
    assert cases.rel_err(got, ref) <= 1e-13


def test_workload_rules_equal_test_restatement():
    """The bench's Yee rules (workloads.yee_linear_rules) are the test's."""
    from masterthesis_gb300 import workloads as W
    for ch in (0.25, 0.5 / np.sqrt(3.0)):
        a, b = W.yee_linear_rules(ch), cases.yee_lin_rules(ch)
        assert a.keys() == b.keys()
        for k in a:
            assert sorted(a[k]) == sorted(b[k]), k


def read_lin_rules(path):
    d = read_device_form(path)
    nu, nph = int(d["lin_cfg"][3]), int(d["lin_cfg"][4])
    r, i, out = d["lin_rules"], 0, {}
    for ph in range(1, nph + 1):
        for f in range(nu):
            for c in range(64):
                k = int(r[i])
                assert r[i + 1] == 0.0
                t = r[i + 2:i + 2 + 5 * k].reshape(k, 5)
                out[(ph, f, c)] = {(int(a), int(b), int(cc), int(dd)): w for a, b, cc, dd, w in t}
                i += 2 + 5 * k
    assert i == len(r)
    return nu, nph, out


@pytest.fixture(scope="module")
def run_problem(native, tmp_path_factory):
    return compile_cpp(HERE / "run_problem.cpp", tmp_path_factory.mktemp("lin") / "run_problem")


def yee_args(n, last, tau, T, fields_path):
    return [f"--nNodes={n[0]}x{n[1]}x{n[2]}", f"--coordNodeLast={last[0]!r}x{last[1]!r}x{last[2]!r}",
            f"--tau={float(tau)!r}", f"--nTimesteps={T}", f"--endtime={float(tau * T)!r}", f"--fields={fields_path}"]


def test_dropin_yee_records_the_yee_rules(run_problem, tmp_path):
    """A Yee class written against the ScaFES callbacks (H in updateInner/
    updateBorder, E in the leapfrog updateInner2/updateBorder2) records
    exactly the Yee rules, for every node class the grid has."""
    n, T = (10, 9, 8), 5
    last, tau, ch, f0 = yee_case(n)
    f0.tofile(tmp_path / "f.bin")
    res = subprocess.run([str(run_problem), "yee", "/dev/null", f"--dump={tmp_path}/d.bin",
                          *yee_args(n, last, tau, T, tmp_path / "f.bin")], capture_output=True, text=True,
                         timeout=120)
    assert res.returncode == 0 and "linear multi-field fields=6 phases=2" in res.stdout, res.stdout + res.stderr
    nu, nph, got = read_lin_rules(tmp_path / "d.bin")
    assert (nu, nph) == (6, 2)
    want = cases.yee_lin_rules(ch)
    present = {c for c in range(64) if all(not ((c >> 2 * p) & 1 and (c >> 2 * p + 1) & 1) for p in range(3))}
    for (ph, f, c), terms in want.items():
        if c not in present:
            continue
        w = {(s, dx, dy, dz): v for s, dx, dy, dz, v in terms}
        assert got[(ph, f, c)].keys() == w.keys(), (ph, f, c)
        for k in w:
            assert got[(ph, f, c)][k] == pytest.approx(w[k], rel=1e-15), (ph, f, c, k)


def test_dropin_refuses_node_varying_multi_field_update(run_problem, tmp_path):
    """A Yee class whose H coefficient differs at one inner node off the
    probed lines: every inner node is checked, and the drop-in refuses the
    problem naming that node (no CPU fallback)."""
    n, T = (10, 9, 8), 5
    last, tau, ch, f0 = yee_case(n)
    f0.tofile(tmp_path / "f.bin")
    res = subprocess.run([str(run_problem), "yee_varying", "/dev/null", "--extract-only",
                          *yee_args(n, last, tau, T, tmp_path / "f.bin")], capture_output=True, text=True,
                         timeout=120)
    assert res.returncode != 0 and "(3,3,3) differs" in res.stderr, res.stdout + res.stderr


def test_lin_create_checks_arguments(native):
    L = native.lib()
    native._lin_bind(L)
    h = C.c_void_p()
    n = (C.c_int * 3)(8, 8, 8)
    assert L.scafes_lin_create(n, 0, 1, None, C.byref(h)) == -1
    assert L.scafes_lin_create(n, 9, 1, None, C.byref(h)) == -1
    assert L.scafes_lin_create(n, 2, 3, None, C.byref(h)) == -1
    assert L.scafes_lin_create((C.c_int * 3)(8, 2, 8), 2, 1, None, C.byref(h)) == -1
    assert L.scafes_lin_create((C.c_int * 3)(8, 8, 65536), 2, 1, None, C.byref(h)) == -1
    assert not h.value
    assert L.scafes_lin_set_rule(None, 1, 0, 0, None, 0, 0.0) == -1
    assert L.scafes_lin_step(None, 1) == -1
    assert L.scafes_lin_upload(None, 0, None, 0) == -1
    L.scafes_lin_destroy(None)
    assert L.scafes_last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [(20, 18, 16), (37, 29, 41)])
def test_linear_yee_matches_oracle(gpu, n):
    M = gpu
    T = 40
    last, tau, ch, f0 = yee_case(n)
    with M.Linear(n, 6, 2) as lin:
        for (ph, f, c), terms in cases.yee_lin_rules(ch).items():
            lin.set_rule(ph, f, c, terms)
        for f in range(6):
            lin.upload(f, f0[f])
        lin.step(T)
        got = np.stack([lin.download(f) for f in range(6)])
        assert lin.last_ms() > 0.0
    ref = O.yee(O.make_grid(n, last=last, tau=tau), f0, T, (0, 0, 0), 0.0, 1.0, 1.0, 1.0)
    assert cases.rel_err(got, ref) <= 1e-12


@pytest.mark.gpu
def test_linear_rule_errors(gpu):
    M = gpu
    n = (8, 8, 8)
    with M.Linear(n, 2, 1) as lin:
        # a class on the x = 0 face has no -x neighbour
        with pytest.raises(M.ScafesError) as e:
            lin.set_rule(1, 0, 1, [(0, -1, 0, 0, 1.0)])
        assert e.value.code == -1
        with pytest.raises(M.ScafesError):
            lin.set_rule(2, 0, 0, [(0, 0, 0, 0, 1.0)])  # one phase only
        with pytest.raises(M.ScafesError):
            lin.set_rule(1, 0, 0, [(2, 0, 0, 0, 1.0)])  # no field 2
        lin.upload(0, np.ones((8, 8, 8)))
        with pytest.raises(M.ScafesError) as e:
            lin.step(1)  # rules missing
        assert e.value.code == -3
        # identity rules everywhere: a step changes nothing
        for f in range(2):
            for c in range(64):
                lin.set_rule(1, f, c, [(f, 0, 0, 0, 1.0)])
        lin.step(3)
        assert np.array_equal(lin.download(0), np.ones((8, 8, 8)))
        assert np.array_equal(lin.download(1), np.zeros((8, 8, 8)))


@pytest.mark.gpu
def test_dropin_yee_matches_oracle(gpu, run_problem, tmp_path):
    """The Yee class through the drop-in's iterateOverTime on the GPU."""
    n, T = (24, 21, 19), 30
    last, tau, ch, f0 = yee_case(n, seed=4)
    f0.tofile(tmp_path / "f.bin")
    out = tmp_path / "out.bin"
    res = subprocess.run([str(run_problem), "yee", str(out), *yee_args(n, last, tau, T, tmp_path / "f.bin")],
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    got = np.fromfile(out, dtype=np.float64).reshape(6, n[2], n[1], n[0])
    ref = O.yee(O.make_grid(n, last=last, tau=tau), f0, T, (0, 0, 0), 0.0, 1.0, 1.0, 1.0)
    assert cases.rel_err(got, ref) <= 1e-12


# The reference's own multi-unknown class: examples/LameNavierEqnFDMFirstOrder
# (six unknown fields, displacements and velocities, coupled through its
# updateInner/updateBorder), compiled unchanged against the drop-in where the
# reference checkout exists; its restatement LameFirstOrder
# (tests/dropin/problems.hpp) must give the same device form byte for byte,
# and runs on the GPU against the reference's own run of the example
# (tests/golden/lame_first_order*.npz, made by
# oracle/ref_harness/ref_lame_first_order.cpp from the untouched headers).
from dropin.build import REFERENCE  # noqa: E402

LAME_FO = REFERENCE / "examples" / "LameNavierEqnFDMFirstOrder"
LAME_FO_GOLDEN = ["lame_first_order", "lame_first_order_b"]


def lame_fo_args(d):
    n = [int(v) for v in d["n"]]
    return [f"--nNodes={n[0]}x{n[1]}x{n[2]}", f"--tau={float(d['tau'])!r}", f"--nTimesteps={int(d['nsteps'])}",
            f"--endtime={float(d['t_end'])!r}"]


@pytest.mark.skipif(not (LAME_FO / "LameNavierEqnFDMFirstOrder.hpp").exists(), reason="reference checkout not present")
@pytest.mark.parametrize("golden", LAME_FO_GOLDEN)
def test_reference_multi_unknown_class_equals_restatement(run_problem, tmp_path, golden):
    from conftest import load_golden
    d = load_golden(golden)
    exe = compile_cpp(HERE / "extract_reference.cpp", tmp_path / "xref11", ["-DPROBLEM=11", "-I", str(LAME_FO)])
    r = subprocess.run([str(exe), f"--dump={tmp_path}/ref.bin", *lame_fo_args(d)], capture_output=True, text=True,
                       timeout=300)
    assert "FORM linear multi-field fields=6 phases=1" in r.stdout, r.stdout + r.stderr
    o = subprocess.run([str(run_problem), "lame_first_order", "/dev/null", f"--dump={tmp_path}/ours.bin",
                        *lame_fo_args(d)], capture_output=True, text=True, timeout=300)
    assert o.returncode == 0, o.stderr
    assert (tmp_path / "ref.bin").read_bytes() == (tmp_path / "ours.bin").read_bytes()


@pytest.mark.gpu
@pytest.mark.parametrize("golden", LAME_FO_GOLDEN)
def test_reference_multi_unknown_class_matches_reference_run(gpu, run_problem, tmp_path, golden):
    """Every unknown field against the reference's run of the example,
    relative max-norm 1e-12 per field (fields that stay zero must stay
    exactly zero)."""
    from conftest import load_golden
    d = load_golden(golden)
    n = [int(v) for v in d["n"]]
    out = tmp_path / "out.bin"
    res = subprocess.run([str(run_problem), "lame_first_order", str(out), *lame_fo_args(d)], capture_output=True,
                         text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    got = np.fromfile(out, dtype=np.float64).reshape(6, n[2], n[1], n[0])
    ref = d["final"]
    for f in range(6):
        if np.max(np.abs(ref[f])) == 0.0:
            assert np.all(got[f] == 0.0), f
        else:
            assert cases.rel_err(got[f], ref[f]) <= 1e-12, f


@pytest.mark.parametrize("golden", LAME_FO_GOLDEN)
def test_recorded_rules_reproduce_reference_run_on_cpu(run_problem, tmp_path, golden):
    """The rules the drop-in records from the restated example, applied on
    the CPU (numpy) from the example's initial state (V3 = omega, the rest
    zero), reproduce the reference's own run: relative max-norm 1e-12 per
    field."""
    from conftest import load_golden
    d = load_golden(golden)
    n = [int(v) for v in d["n"]]
    o = subprocess.run([str(run_problem), "lame_first_order", "/dev/null", f"--dump={tmp_path}/d.bin",
                        *lame_fo_args(d)], capture_output=True, text=True, timeout=300)
    assert o.returncode == 0, o.stderr
    nu, nph, rules = read_lin_rules(tmp_path / "d.bin")
    assert (nu, nph) == (6, 1)
    terms = {k: [(s, dx, dy, dz, w) for (s, dx, dy, dz), w in v.items()] for k, v in rules.items()}
    f0 = np.zeros((6, n[2], n[1], n[0]))
    f0[5] = 2.0 * np.pi
    got = apply_rules(terms, f0, 1, int(d["nsteps"]))
    ref = d["final"]
    for f in range(6):
        if np.max(np.abs(ref[f])) == 0.0:
            assert np.all(got[f] == 0.0), f
        else:
            assert cases.rel_err(got[f], ref[f]) <= 1e-12, f


@pytest.mark.gpu
def test_linear_smallest_grid_and_most_fields(gpu):
    """A 3 x 3 x 3 grid (one inner node; corner, edge and face classes) with
    SCAFES_LIN_MAX_FIELDS fields: each field takes the rule
    u' = 2u + 0.5 * (next field at the same node) on every class, checked
    against numpy after 3 steps, bit for bit."""
    M = gpu
    n, nf = (3, 3, 3), M.LIN_MAX_FIELDS
    rng = np.random.default_rng(12)
    f0 = rng.uniform(-1.0, 1.0, (nf, 3, 3, 3))
    with M.Linear(n, nf, 1) as lin:
        for f in range(nf):
            for c in range(64):
                lin.set_rule(1, f, c, [(f, 0, 0, 0, 2.0), ((f + 1) % nf, 0, 0, 0, 0.5)])
            lin.upload(f, f0[f])
        lin.step(3)
        got = np.stack([lin.download(f) for f in range(nf)])
    # 2u and 0.5v are exact, so the kernel's FMA and numpy's sum round alike.
    want = f0.copy()
    for _ in range(3):
        want = np.stack([2.0 * want[f] + 0.5 * want[(f + 1) % nf] for f in range(nf)])
    assert np.array_equal(got, want)
