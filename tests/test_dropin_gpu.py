"""The C++ drop-in ScaFES::Problem on the GPU: problem classes written
against the ScaFES callback interface run iterateOverTime() through the C
ABI and reproduce the reference's golden vectors (relative max-norm 1e-12)."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

import cases
import oracle as O
from conftest import load_golden
from dropin.build import HERE, compile_cpp

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def run_problem(gpu, tmp_path_factory):
    return compile_cpp(HERE / "run_problem.cpp", tmp_path_factory.mktemp("dropin_gpu") / "run_problem")


def run(exe, name, out, n, *opts):
    res = subprocess.run([str(exe), name, str(out), *opts], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    return np.fromfile(out, dtype=np.float64).reshape(n[2], n[1], n[0]), res.stdout


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
@pytest.mark.parametrize("name,golden", [("heat_lin", "heat_timelin"), ("pennes_lin", "pennes_timelin")])
def test_dropin_timelin_matches_reference(run_problem, tmp_path, name, golden, prec):
    d = load_golden(golden)
    n = tuple(int(v) for v in d["n"])
    u, out = run(run_problem, name, tmp_path / "u.bin", n, f"--nNodes={n[0]}x{n[1]}x{n[2]}",
                 f"--nTimesteps={int(d['nsteps'])}", f"--endtime={float(d['t_end'])!r}", f"--gpuPrecision={prec}")
    assert cases.rel_err(u, d["final"]) <= 1e-12
    assert "Local Linf error" in out


def test_dropin_stencil_width_one_matches_reference(run_problem, tmp_path):
    d = load_golden("stencil_width_one")
    n = tuple(int(v) for v in d["n"])
    u, _ = run(run_problem, "mirror_pow2", tmp_path / "u.bin", n, "--nNodes=32x32x32", "--nTimesteps=20",
               "--coordNodeLast=1000x1000x1000", "--gpuAutotune=1")
    assert cases.rel_err(u, d["final"]) <= 1e-12


def test_dropin_heat_sine_config1_vs_oracle(run_problem, tmp_path):
    n, T = (64, 64, 64), 200
    h = 1.0 / 63
    tau = 0.9 * h * h / 6.0
    u, _ = run(run_problem, "heat_sine", tmp_path / "u.bin", n, "--nNodes=64x64x64", f"--nTimesteps={T}",
               f"--tau={tau!r}")
    g = O.make_grid(n, tau=tau)
    x, y, z = O.coords(g)
    u0 = np.broadcast_to(np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z), (64, 64, 64)).copy()
    u0[O.border_mask(g)] = 0.0
    ref = O.heat_dirichlet(g, u0, T)
    assert cases.rel_err(u, ref) <= 1e-12


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
@pytest.mark.parametrize("name,golden", [("heat_neumann", "heat_neumann"), ("heat_cauchy", "heat_cauchy"),
                                         ("heat_neumann", "heat_neumann_10x8x6")])
def test_dropin_flux_border_matches_reference(run_problem, tmp_path, name, golden, prec):
    """Neumann / Cauchy border problems through the drop-in Problem: the
    border rules are extracted per border class and run as a rule table."""
    d = load_golden(golden)
    n = tuple(int(v) for v in d["n"])
    u, out = run(run_problem, name, tmp_path / "u.bin", n, f"--nNodes={n[0]}x{n[1]}x{n[2]}",
                 f"--nTimesteps={int(d['nsteps'])}", f"--endtime={float(d['t_end'])!r}", f"--gpuPrecision={prec}")
    assert cases.rel_err(u, d["final"]) <= 1e-12


@pytest.mark.parametrize("prec", ["f64", "f32x2"])
@pytest.mark.parametrize("golden", ["pennes_radiation", "pennes_radiation_10x8x6"])
def test_dropin_radiation_border_matches_reference(run_problem, tmp_path, golden, prec):
    """The radiation border through the drop-in Problem: the u^4 flux is
    recorded into the rule table and the quartic-in-time border field is
    fitted in the device's time basis; against the reference's own final
    iterate of Radiation/TimeLinSpaceLin."""
    d = load_golden(golden)
    n = tuple(int(v) for v in d["n"])
    u, out = run(run_problem, "pennes_radiation", tmp_path / "u.bin", n, f"--nNodes={n[0]}x{n[1]}x{n[2]}",
                 f"--nTimesteps={int(d['nsteps'])}", f"--endtime={float(d['t_end'])!r}", f"--gpuPrecision={prec}")
    assert cases.rel_err(u, d["final"]) <= 1e-12


@pytest.mark.parametrize("name,golden", [("heat_lin", "heat_timelin_nl2"), ("heat_neumann", "heat_neumann_nl3"),
                                         ("pennes_radiation", "pennes_radiation_nl2")])
def test_dropin_border_layers_match_reference(run_problem, tmp_path, name, golden):
    """--nLayersAtBorder=2/3: the drop-in classifies border nodes by layer
    and records a rule for the border nodes on no face (class 0)."""
    d = load_golden(golden)
    n = tuple(int(v) for v in d["n"])
    u, out = run(run_problem, name, tmp_path / "u.bin", n, f"--nNodes={n[0]}x{n[1]}x{n[2]}",
                 f"--nTimesteps={int(d['nsteps'])}", f"--endtime={float(d['t_end'])!r}",
                 f"--nLayersAtBorder={int(d['n_layers'])}", "--gpuPrecision=f64")
    assert cases.rel_err(u, d["final"]) <= 1e-12


def test_dropin_writes_snapshots_like_given_at_cl(gpu, run_problem, tmp_path):
    """writeToFile = LIKE_GIVEN_AT_CL with --nSnapshots=3 over 300 steps
    writes the unknown field at steps 0, 100, 200 and 300 (the reference's
    nTimesteps/nSnapshots rule); the last one is the final iterate."""
    M = gpu
    d = load_golden("heat_timelin")
    n = tuple(int(v) for v in d["n"])
    snap = tmp_path / "u.snap"
    u, _ = run(run_problem, "heat_lin", tmp_path / "u.bin", n, f"--nNodes={n[0]}x{n[1]}x{n[2]}",
               f"--nTimesteps={int(d['nsteps'])}", f"--endtime={float(d['t_end'])!r}", "--nSnapshots=3",
               f"--gpuSnapshotFile={snap}", "--write-like-cl")
    assert M.snapshot_info(snap) == (n, 4)
    steps = [M.snapshot_read(snap, k)[1] for k in range(4)]
    assert steps == [0, 100, 200, 300]
    assert np.array_equal(M.snapshot_read(snap, 3)[0], u)
    assert cases.rel_err(u, d["final"]) <= 1e-12


def test_dropin_restarts_from_init_file(gpu, run_problem, tmp_path):
    """--initfile (the reference's restart: evalInitPbPhase reads the
    unknown fields from a file instead of calling initInner/initBorder):
    a run of the last 200 steps started from the snapshot at step 100 of a
    300-step run, with --starttime at that step's time, ends where the full
    run ends (1e-12; tau is recomputed from the shorter interval, so the
    last bits may differ).  A missing or mismatched file is refused."""
    d = load_golden("heat_timelin")
    n = tuple(int(v) for v in d["n"])
    snap = tmp_path / "u.snap"
    full, _ = run(run_problem, "heat_lin", tmp_path / "u.bin", n, f"--nNodes={n[0]}x{n[1]}x{n[2]}",
                  "--nTimesteps=300", "--endtime=1.0", "--nSnapshots=3", f"--gpuSnapshotFile={snap}",
                  "--write-like-cl")
    t100 = 100 * (1.0 / 300)
    part, out = run(run_problem, "heat_lin", tmp_path / "v.bin", n, f"--nNodes={n[0]}x{n[1]}x{n[2]}",
                    "--nTimesteps=200", f"--starttime={t100!r}", "--endtime=1.0", f"--initfile={snap}",
                    "--initfileIndex=1")
    assert cases.rel_err(part, full) <= 1e-12
    res = subprocess.run([str(run_problem), "heat_lin", str(tmp_path / "w.bin"), "--nNodes=9x8x8",
                          "--nTimesteps=10", f"--initfile={snap}"], capture_output=True, text=True, timeout=120)
    assert res.returncode != 0 and "another grid" in (res.stdout + res.stderr)
    res = subprocess.run([str(run_problem), "heat_lin", str(tmp_path / "w.bin"), f"--nNodes={n[0]}x{n[1]}x{n[2]}",
                          "--nTimesteps=10", f"--initfile={tmp_path / 'missing.snap'}"],
                         capture_output=True, text=True, timeout=120)
    assert res.returncode != 0 and "init file" in (res.stdout + res.stderr)


@pytest.mark.parametrize("prec,tol", [("f64", 1e-12), ("f32", 1e-5)])
@pytest.mark.parametrize("which,golden", [("tumour", "tissue_tumour"), ("mri", "tissue_mri_closed")])
def test_dropin_tissue_examples_match_reference(run_problem, tmp_path, which, golden, prec, tol):
    """The tissue examples (coefficients per node, per-node flux borders)
    through iterateOverTime on the variable-coefficient sweep, against the
    reference's own classes run by its driver (tests/golden/tissue_*.npz).
    The restatements' device forms equal the reference classes' bit for bit
    (test_dropin_host.py)."""
    from dropin.build import tissue_args
    d = load_golden(golden)
    n = tuple(int(v) for v in d["n"])
    u, out = run(run_problem, which, tmp_path / "u.bin", n, *tissue_args(d, tmp_path), f"--gpuPrecision={prec}")
    assert cases.rel_err(u, d["final"]) <= tol
