"""The C++ drop-in ScaFES::Problem without a GPU: problem classes written
against the ScaFES callback interface compile against the drop-in headers,
and the stencil extraction maps their updates to the expected device form
(or refuses them with a message).  Where the reference checkout exists, the
reference's own system-test classes are compiled unchanged and checked the
same way."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

import numpy as np

from conftest import load_golden
from dropin.build import HERE, REFERENCE, compile_cpp, read_device_form, tissue_args


@pytest.fixture(scope="module")
def run_problem(native, tmp_path_factory):
    return compile_cpp(HERE / "run_problem.cpp", tmp_path_factory.mktemp("dropin") / "run_problem")


def form(exe, *args):
    out = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    return out.stdout


@pytest.mark.parametrize("name,expect", [
    ("heat_lin", ["c0=0.02 ", "cp=(0.163333,0.163333,0.163333)", "source=static", "border=dirichlet"]),
    ("pennes_lin", ["c0=0.0166667", "source=affine", "border=dirichlet"]),
    ("mirror_pow2", ["c0=0.285714", "source=none", "border=mirror"]),
    ("heat_neumann", ["c0=0.02 ", "source=static", "border=table"]),
    ("heat_cauchy", ["c0=0.02 ", "source=static", "border=table"]),
    ("pennes_radiation", ["source=affine", "border=table", "G=quartic-in-time", "u^4"]),
])
def test_extracted_form(run_problem, name, expect):
    s = form(run_problem, name, "/dev/null", "--extract-only", "--nNodes=8x8x8", "--nTimesteps=300", "--endtime=1")
    for e in expect:
        assert e in s, s


REF_SYS = REFERENCE / "tests" / "system"
REF_CASES = [
    (1, ["HeatEqnFDM", "HeatEqnFDM/Dirichlet", "HeatEqnFDM/Dirichlet/TimeLinSpaceLin"], "FORM star7 c0=0.02 ", "border=dirichlet"),
    (2, ["PennesBioheatEqnFDM", "PennesBioheatEqnFDM/Dirichlet", "PennesBioheatEqnFDM/Dirichlet/TimeLinSpaceLin"],
     "source=affine", "border=dirichlet"),
    (3, ["HeatEqnFdmStencilWidthOne"], "c0=0.285714", "border=mirror"),
    (4, ["HeatEqnFDM", "HeatEqnFDM/Neumann", "HeatEqnFDM/Neumann/TimeLinSpaceLin"], "FORM star7 c0=0.02 ",
     "border=table"),
    (6, ["HeatEqnFDM", "HeatEqnFDM/Cauchy", "HeatEqnFDM/Cauchy/TimeLinSpaceLin"], "FORM star7 c0=0.02 ",
     "border=table"),
    (7, ["PennesBioheatEqnFDM", "PennesBioheatEqnFDM/Neumann", "PennesBioheatEqnFDM/Neumann/TimeLinSpaceLin"],
     "source=affine", "border=table"),
    (8, ["PennesBioheatEqnFDM", "PennesBioheatEqnFDM/Radiation",
         "PennesBioheatEqnFDM/Radiation/TimeLinSpaceLin"], "border=table G=quartic-in-time u^4", "source=affine"),
    (5, ["PropagationFromLeftLowerCorner"], "REFUSED", "branches on the value"),
]


@pytest.mark.skipif(not (REF_SYS / "HeatEqnFDM").exists(), reason="reference checkout not present")
@pytest.mark.parametrize("pid,dirs,e1,e2", REF_CASES)
def test_reference_system_test_classes_unchanged(native, tmp_path, pid, dirs, e1, e2):
    extra = [f"-DPROBLEM={pid}"] + sum((["-I", str(REF_SYS / d)] for d in dirs), [])
    exe = compile_cpp(HERE / "extract_reference.cpp", tmp_path / f"xref{pid}", extra)
    s = form(exe, "--nNodes=8x8x8", "--nTimesteps=300", "--endtime=1")
    assert e1 in s and e2 in s, s


# Each restatement of tests/dropin/problems.hpp against the reference class it
# restates: the whole device form (configuration, border rules, every field
# the device run uploads) must be equal bit for bit, so the GPU runs of the
# restatements execute the reference classes' own updates.
PAIRS = [
    (1, "heat_lin", ["HeatEqnFDM", "HeatEqnFDM/Dirichlet", "HeatEqnFDM/Dirichlet/TimeLinSpaceLin"]),
    (2, "pennes_lin", ["PennesBioheatEqnFDM", "PennesBioheatEqnFDM/Dirichlet",
                       "PennesBioheatEqnFDM/Dirichlet/TimeLinSpaceLin"]),
    (3, "mirror_pow2", ["HeatEqnFdmStencilWidthOne"]),
    (4, "heat_neumann", ["HeatEqnFDM", "HeatEqnFDM/Neumann", "HeatEqnFDM/Neumann/TimeLinSpaceLin"]),
    (6, "heat_cauchy", ["HeatEqnFDM", "HeatEqnFDM/Cauchy", "HeatEqnFDM/Cauchy/TimeLinSpaceLin"]),
    (8, "pennes_radiation", ["PennesBioheatEqnFDM", "PennesBioheatEqnFDM/Radiation",
                             "PennesBioheatEqnFDM/Radiation/TimeLinSpaceLin"]),
]


def same_device_form(ref_exe, ours_exe, which, args, tmp):
    r = subprocess.run([str(ref_exe), f"--dump={tmp}/ref.bin", *args], capture_output=True, text=True, timeout=300)
    o = subprocess.run([str(ours_exe), which, "/dev/null", f"--dump={tmp}/ours.bin", *args], capture_output=True,
                       text=True, timeout=300)
    assert "FORM" in r.stdout and "FORM" in o.stdout, (r.stdout, o.stdout, o.stderr)
    a, b = read_device_form(tmp / "ref.bin"), read_device_form(tmp / "ours.bin")
    assert a.keys() == b.keys()
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert (tmp / "ref.bin").read_bytes() == (tmp / "ours.bin").read_bytes()
    return r.stdout


@pytest.mark.skipif(not (REF_SYS / "HeatEqnFDM").exists(), reason="reference checkout not present")
@pytest.mark.parametrize("pid,which,dirs", PAIRS)
def test_restatement_equals_reference_class(run_problem, tmp_path, pid, which, dirs):
    extra = [f"-DPROBLEM={pid}"] + sum((["-I", str(REF_SYS / d)] for d in dirs), [])
    exe = compile_cpp(HERE / "extract_reference.cpp", tmp_path / f"xref{pid}", extra)
    same_device_form(exe, run_problem, which, ["--nNodes=8x8x8", "--nTimesteps=300", "--endtime=1"], tmp_path)


STUB = HERE.parents[1] / "oracle" / "ref_harness" / "stub"   # Boost.PropertyTree stand-in


@pytest.mark.skipif(not (REFERENCE / "examples" / "TumorHeatEqnFDM").exists(), reason="reference checkout not present")
@pytest.mark.parametrize("pid,which,golden,exdir", [
    (9, "tumour", "tissue_tumour", "TumorHeatEqnFDM"),
    (10, "mri", "tissue_mri_closed", "MRIDataPBHEqnFDM"),
])
def test_tissue_restatement_equals_reference_example(run_problem, tmp_path, pid, which, golden, exdir):
    """The reference's tissue examples, compiled unchanged against the
    drop-in, map to the variable-coefficient sweep with per-node border
    rules -- the same device form as their restatements, which the GPU tests
    run against the reference's own golden vectors."""
    exe = compile_cpp(HERE / "extract_reference.cpp", tmp_path / f"xref{pid}",
                      [f"-DPROBLEM={pid}", "-I", str(STUB), "-I", str(REFERENCE / "examples" / exdir)])
    out = same_device_form(exe, run_problem, which, tissue_args(load_golden(golden), tmp_path), tmp_path)
    assert "star7-vc" in out and "border=nodes" in out, out


@pytest.mark.skipif(not (REFERENCE / "examples" / "MRIDataPBHEqnFDM").exists(), reason="reference checkout not present")
def test_open_skull_radiation_is_refused(run_problem, tmp_path):
    """Where the MRI example's skull is open its z-max face radiates with the
    fourth power of the partially updated node value -- not linear in the
    old iterate -- and the drop-in refuses it (no CPU fallback), for the
    reference class and its restatement alike."""
    args = tissue_args(load_golden("tissue_mri_open"), tmp_path)
    exe = compile_cpp(HERE / "extract_reference.cpp", tmp_path / "xref10",
                      ["-DPROBLEM=10", "-I", str(STUB), "-I", str(REFERENCE / "examples" / "MRIDataPBHEqnFDM")])
    r = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=300)
    assert "REFUSED" in r.stdout and "not a linear stencil" in r.stdout, r.stdout
    o = subprocess.run([str(run_problem), "mri", "/dev/null", "--extract-only", *args], capture_output=True,
                       text=True, timeout=300)
    assert o.returncode != 0 and "not linear" in o.stderr, o.stderr


def test_tissue_restatements_map_to_vc(run_problem, tmp_path):
    """Without the reference checkout: the tissue restatements map to the
    variable-coefficient sweep with per-node border rules."""
    for which, golden in (("tumour", "tissue_tumour"), ("mri", "tissue_mri_closed")):
        s = form(run_problem, which, "/dev/null", "--extract-only", *tissue_args(load_golden(golden), tmp_path))
        assert "star7-vc" in s and "source=static" in s and "border=nodes" in s, s
